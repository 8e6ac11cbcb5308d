/*
 * mks_oracle.c — serial CPU restatement of the MulSKIPS KMC program.
 *
 * TEST INFRASTRUCTURE ONLY (see mks_oracle.h).  This file restates the
 * reference Fortran, routine by routine, on the same dense int32 bit-field
 * grid.  Every routine cites the reference file:line it follows.  Paths are
 * relative to the MulSKIPS project root; MS/ = mulskips-source/.
 *
 * Bit-exactness notes (all mirror the compiled reference):
 *  - ran3 `fac` is the single-precision quotient 1./1e9 widened to double
 *    (MS/mcevent/random.f:24,29).
 *  - the test-mode uniforms are single-precision literals widened to double
 *    (MS/mcevent/PickTreeEvent.f:77-1076); they are loaded from a fixture.
 *  - the dummy rate of unsupported coor-1 sites is the single-precision
 *    literal 1.e-8 (MS/mcevent/Get_Prob.f:183); Pi in FIND_NN is the
 *    single-precision literal widened (MS/lattice/FIND_NN.f:27); the
 *    arm-chair shift 8.6602254037 is single precision (FIND_SN.f:67).
 *  - sum-tree parents are left+right recomputed bottom-up
 *    (MS/mcevent/UpdateTree.f:49-65).
 * Out-of-range reads that the Fortran performs silently (z<0 neighbours of a
 * z=0 bulk layer, list index 0) read zero-filled guard storage here.
 */
#include "mks_oracle.h"

#include <math.h>
#include <setjmp.h>
#include <stdarg.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <ctype.h>

/* ---- bit layout, MS/modules/defsystem.f:87-91 ---- */
#define POS_INDEX 0
#define LEN_INDEX 8
#define POS_T 9
#define LEN_T 13
#define POS_OCC 23
#define LEN_OCC 1
#define POS_COOR 24
#define LEN_COOR 3
#define POS_SIC 27
#define LEN_SIC 3
#define POS_SI 27
#define POS_C 28
#define WALL 113

#define NCRYSTAL_MAX 3
#define NCOV_MAX 3
#define ZGUARD 8          /* zero planes below z=0 and above z=LenZ */

typedef struct {
    int xyz[3];
    int nn[4][3];
    int ind_event;
    double prob;
} mcp_t;                  /* MCParticle, MS/modules/defdertype.f:32-37 */

typedef struct {
    int xyz[3];
    int nn[4][3];
} blk_t;                  /* BulkParticle / Vacancy, defdertype.f:25-45 */

typedef struct {
    int xyz[3];
    int ind_atype;
} atbuf_t;                /* AtBuffer, defdertype.f:47-50 */

/* ran3 (MS/mcevent/random.f:22-69) */
typedef struct {
    int ma[56];
    int inext, inextp, iff;
} ran3_t;

struct ora {
    int lx, ly, lz;
    int32_t *latt_base, *latt;     /* LattCoo(0:lx-1,0:ly-1,0:lz) */
    int32_t *lind_base, *lind;     /* LattInd */
    /* lists (1-based, element 0 is a zero guard) */
    mcp_t *mc; int num_mc, mc_max;          /* ListAdAtom, NumMcMax */
    blk_t *bulk; int64_t num_bulk, bulk_cap, bulk_max;   /* ListAtom */
    blk_t *voids; int num_void, void_max;   /* ListVoid */
    atbuf_t *atbuf; int atbuf_cap;
    double *tree; int levels, size_tree;
    /* model */
    int ncrystal, ncov;
    int list_crystal[NCRYSTAL_MAX], list_cov[NCOV_MAX];
    int count_crystal[NCRYSTAL_MAX], count_crystal_old[NCRYSTAL_MAX];
    int count_cov[NCOV_MAX];
    double ptransE[NCRYSTAL_MAX][4][4][4][4][4][4];
    double ptransD[NCRYSTAL_MAX][3];
    double ptransAbs[NCOV_MAX][4], ptransDes[NCOV_MAX][4];
    double ptrans_zig;
    double sf;
    double alloyfraction;
    /* LA law parameters (MS/modules/definitions.f:30) and the LA start.dat
     * block (MS/main.f:118-138) */
    double Tm, P0, sigma, Tflex;
    double len_vac, len_nuc;
    char homogeneous[3];
    /* per-species LA law with liquid fractions and the LR score (ora_la_*) */
    int la2;
    ora_la_t lap;
    double dE[NCRYSTAL_MAX][4][4][4][4];    /* d PTransE(s,n1,n2,n3,0,0,0) / d theta_j */
    double dEd[NCRYSTAL_MAX][3][4];         /* d PTransD(s,n) / d theta_j              */
    double xliq[3];
    int64_t la_init[3], la_cnt[3], la_win, la_events;
    double la_score[4];
    uint64_t la_rng[4];
    int la_stop;
    double *la_k, *la_dk, *la_ps;           /* per-MC-particle rates of the last scan */
    int *la_kind, la_cap;
    int la_cur_z;                           /* grid z of the site whose rate la2_pd evaluates */
    int8_t *la_geo;                         /* InitSt LA input (ora_set_la_input) */
    int16_t *la_tsub;
    int8_t *cad_geo;                        /* InitSt IN input (ora_set_geometry) */
    char shapefile[2048];                   /* InitSt SH: the point-list file named in start.dat */
    /* InitSt ST: probability tables per temperature (SetProbabilityFromField.f)
     * and the interpolation pair of the last site (InterpProbFromField.f) */
    int st, st_fixed, st_n;
    int st_T[300];
    double (*st_E)[NCRYSTAL_MAX][4][4][4][4][4][4];
    double (*st_D)[NCRYSTAL_MAX][3];
    double st_angle, st_ttop, st_tbottom;
    int st_lo, st_hi, st_wl, st_wu;
    char init_st[3], run_type[3], exit_strategy[5];
    char save_final[3], save_coo[3];
    char restartfile[2048], coofile[2048];
    int len1, len2, len3, len4;
    int64_t max_iter, out_molmol;
    double max_time, out_time;
    int idum;
    ran3_t rng;
    int counter;                    /* test-mode list counter */
    double numbers[1000];
    int have_numbers;
    /* loop state (MS/main.f:31-54) */
    int64_t iter, iter_out, framecounter;
    double time;
    int started;
    /* Evaporation's NBuff: a local of Evaporation.f:33 that is read even
     * when not assigned in the same call; kept across calls here. */
    int nbuff[3];
    /* trace */
    int trace_on;
    ora_event_t *trace; int64_t trace_len, trace_cap;
    int cur_arm;
    /* log */
    FILE *log;
    jmp_buf jb;
    char err[512];
};

static char g_err[512];
const char *ora_last_error(void) { return g_err; }

static void ora_fail(ora_t *o, const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(o->err, sizeof o->err, fmt, ap);
    va_end(ap);
    snprintf(g_err, sizeof g_err, "%s", o->err);
    longjmp(o->jb, 1);
}

static void lg(ora_t *o, const char *fmt, ...)
{
    if (!o->log) return;
    va_list ap;
    va_start(ap, fmt);
    vfprintf(o->log, fmt, ap);
    va_end(ap);
}

/* ---- bit helpers: IBITS / MVBITS ---- */
static inline int ibits(int32_t v, int pos, int len)
{
    return (int)(((uint32_t)v >> pos) & ((1u << len) - 1u));
}
static inline void mvbits(int from, int len, int32_t *to, int pos)
{
    uint32_t m = ((1u << len) - 1u) << pos;
    *to = (int32_t)(((uint32_t)*to & ~m) | (((uint32_t)from << pos) & m));
}

static inline int64_t lidx(const ora_t *o, int x, int y, int z)
{
    return (int64_t)x + (int64_t)o->lx * ((int64_t)y + (int64_t)o->ly * (int64_t)z);
}
static inline int32_t *LC(ora_t *o, const int s[3]) { return &o->latt[lidx(o, s[0], s[1], s[2])]; }
static inline int32_t *LI(ora_t *o, const int s[3]) { return &o->lind[lidx(o, s[0], s[1], s[2])]; }
static inline int same3(const int a[3], const int b[3]) { return a[0] == b[0] && a[1] == b[1] && a[2] == b[2]; }
static inline void cp3(int d[3], const int s[3]) { d[0] = s[0]; d[1] = s[1]; d[2] = s[2]; }

/* JumpDia, MS/modules/defsystem.f:104-105 (bond vectors of the two fcc
 * sublattices; columns 1-4 for (x1+y1+z1) mod 4 == 0 sites, 5-8 for == 3). */
static const int JUMPDIA[8][3] = {
    {3, 3, 3}, {3, -3, -3}, {-3, -3, 3}, {-3, 3, -3},
    {3, 3, -3}, {3, -3, 3}, {-3, -3, -3}, {-3, 3, 3}};

/* ================= RNG: ran3, MS/mcevent/random.f:22-69 ================= */
#define MBIG 1000000000
#define MSEED 161803398
#define MZ 0
static double ran3_fac(void)
{
    volatile float f = 1.0f / (float)MBIG;   /* fac=1./Mbig, default real */
    return (double)f;
}
static double ran3(ran3_t *r, int *idum)
{
    int mj, mk, i, ii, k;
    if (*idum < 0 || r->iff == 0) {
        r->iff = 1;
        mj = MSEED - abs(*idum);
        mj = mj % MBIG;
        r->ma[55] = mj;
        mk = 1;
        for (i = 1; i <= 54; i++) {
            ii = (21 * i) % 55;
            r->ma[ii] = mk;
            mk = mj - mk;
            if (mk < MZ) mk += MBIG;
            mj = r->ma[ii];
        }
        for (k = 1; k <= 4; k++)
            for (i = 1; i <= 55; i++) {
                r->ma[i] = r->ma[i] - r->ma[1 + (i + 30) % 55];
                if (r->ma[i] < MZ) r->ma[i] += MBIG;
            }
        r->inext = 0;
        r->inextp = 31;
        *idum = 1;
    }
    r->inext++;
    if (r->inext == 56) r->inext = 1;
    r->inextp++;
    if (r->inextp == 56) r->inextp = 1;
    mj = r->ma[r->inext] - r->ma[r->inextp];
    if (mj < MZ) mj += MBIG;
    r->ma[r->inext] = mj;
    return (double)mj * ran3_fac();
}
static double rnd(ora_t *o) { return ran3(&o->rng, &o->idum); }

void ora_ran3_sequence(int idum, int n, double *out)
{
    ran3_t r;
    memset(&r, 0, sizeof r);
    for (int i = 0; i < n; i++) out[i] = ran3(&r, &idum);
}

/* ============ sum-tree: MS/mcevent/UpdateTree.f:25-66 ============ */
static void update_tree(ora_t *o, int index, double patom)
{
    if (patom == 0.0 && index < o->num_mc)
        ora_fail(o, "error stabilizzato da dentro Update! %d", index);
    else if (index > o->num_mc)
        ora_fail(o, "Index > NumAdAtom %d %d", index, o->num_mc);
    int pos = index + (1 << (o->levels - 1)) - 1;
    o->tree[pos] = patom;
    for (int parent = o->levels - 1; parent >= 1; parent--) {
        int neigh = (pos & 1) ? pos - 1 : pos + 1;
        int np = pos >> 1;
        o->tree[np] = o->tree[pos] + o->tree[neigh];
        pos = np;
    }
}

/* AllocateArrays, MS/mcevent/AllocateArrays.f:24-45 */
static void allocate_arrays(ora_t *o)
{
    int lev = 0;
    for (int ind = 0; ind <= 31; ind++)
        if ((o->mc_max >> ind) & 1) lev = ind;
    if (o->mc_max > (1 << lev)) lev += 2; else lev += 1;
    o->levels = lev;
    o->size_tree = (1 << lev) - 1;
    free(o->tree);
    o->tree = (double *)calloc((size_t)o->size_tree + 2, sizeof(double));
    if (!o->tree) ora_fail(o, "tree allocation failed");
    lg(o, " numParticelle= %d Levels = %d , SizeTree = %d\n", o->mc_max, o->levels, o->size_tree);
}

/* PickTreeEvent, MS/mcevent/PickTreeEvent.f:25-70 */
static int pick_tree_event(ora_t *o, double *patom)
{
    int index = 1;
    for (int parent = 1; parent <= o->levels - 1; parent++) {
        double u;
        if (o->run_type[0] == 'T') {
            o->counter++;
            u = o->numbers[(o->counter - 1) % 1000];
        } else {
            u = rnd(o);
        }
        *patom = u * o->tree[index];
        index <<= 1;
        if (o->tree[index] < *patom) index++;
    }
    *patom = o->tree[index];
    if (index - (1 << (o->levels - 1)) + 1 > o->num_mc)
        ora_fail(o, "write Index> NumAdAtom");
    return index - (1 << (o->levels - 1)) + 1;
}

/* ============ lists: MS/mcevent/Add.f, Erase.f ============ */
static void add_mc(ora_t *o, const int site[3], int nextn[4][3], int ind_event, double prob)
{   /* Add.f:24-52 */
    if (prob == 0.0) ora_fail(o, "provo ad aggiungere prob nulla");
    o->num_mc++;
    if (o->num_mc >= o->mc_max) ora_fail(o, "troppe particelle cinetiche %d", o->num_mc);
    *LI(o, site) = o->num_mc;
    mcp_t *p = &o->mc[o->num_mc];
    cp3(p->xyz, site);
    memcpy(p->nn, nextn, sizeof p->nn);
    p->ind_event = ind_event;
    p->prob = prob;
    update_tree(o, o->num_mc, prob);
}

static void add_bulk(ora_t *o, const int site[3], int nextn[4][3])
{   /* Add.f:57-76 */
    o->num_bulk++;
    if (o->num_bulk >= o->bulk_max) ora_fail(o, "troppe particelle bulk");
    if (o->num_bulk >= o->bulk_cap) {
        int64_t nc = o->bulk_cap * 2;
        blk_t *nb = (blk_t *)realloc(o->bulk, (size_t)nc * sizeof(blk_t));
        if (!nb) ora_fail(o, "bulk list allocation failed");
        memset(nb + o->bulk_cap, 0, (size_t)(nc - o->bulk_cap) * sizeof(blk_t));
        o->bulk = nb;
        o->bulk_cap = nc;
    }
    *LI(o, site) = (int32_t)o->num_bulk;
    cp3(o->bulk[o->num_bulk].xyz, site);
    memcpy(o->bulk[o->num_bulk].nn, nextn, sizeof(int) * 12);
}

static void add_void(ora_t *o, const int site[3], int nextn[4][3])
{   /* Add.f:82-101 */
    o->num_void++;
    if (o->num_void >= o->void_max) ora_fail(o, "troppe vacanze");
    *LI(o, site) = o->num_void;
    cp3(o->voids[o->num_void].xyz, site);
    memcpy(o->voids[o->num_void].nn, nextn, sizeof(int) * 12);
}

static void erase_mc(ora_t *o, const int site[3])
{   /* Erase.f:24-76 */
    if (site[2] == -1) ora_fail(o, "accesso a latt fuori bond");
    int ind = *LI(o, site);
    if (ind > o->mc_max || ind == 0) ora_fail(o, "err: EraseMC %d %d %d %d", ind, site[0], site[1], site[2]);
    if (ind >= o->num_mc) {
        memset(&o->mc[ind], 0, sizeof(mcp_t));
        *LI(o, site) = 0;
        update_tree(o, ind, 0.0);
        o->num_mc--;
    } else {
        o->mc[ind] = o->mc[o->num_mc];
        int leaf = o->num_mc + (1 << (o->levels - 1)) - 1;
        update_tree(o, ind, o->tree[leaf]);
        update_tree(o, o->num_mc, 0.0);
        int st[3];
        cp3(st, o->mc[o->num_mc].xyz);
        *LI(o, st) = ind;
        memset(&o->mc[o->num_mc], 0, sizeof(mcp_t));
        *LI(o, site) = 0;
        o->num_mc--;
    }
}

static void erase_bulk(ora_t *o, const int site[3])
{   /* Erase.f:82-127 */
    if (site[2] == -1) ora_fail(o, "accesso a latt fuori bond");
    int64_t ind = *LI(o, site);
    if (ind > o->bulk_max || ind == 0) ora_fail(o, "err: EraseBulk");
    if (ind == o->num_bulk) {
        memset(&o->bulk[o->num_bulk], 0, sizeof(blk_t));
        *LI(o, site) = 0;
        o->num_bulk--;
    } else {
        o->bulk[ind] = o->bulk[o->num_bulk];
        int st[3];
        cp3(st, o->bulk[o->num_bulk].xyz);
        *LI(o, st) = (int32_t)ind;
        memset(&o->bulk[o->num_bulk], 0, sizeof(blk_t));
        *LI(o, site) = 0;
        o->num_bulk--;
    }
}

static void erase_void(ora_t *o, const int site[3])
{   /* Erase.f:134-179 */
    if (site[2] == -1) ora_fail(o, "accesso a latt fuori bond");
    int ind = *LI(o, site);
    if (ind > o->void_max || ind == 0) ora_fail(o, "err: EraseVoid");
    if (ind == o->num_void) {
        memset(&o->voids[o->num_void], 0, sizeof(blk_t));
        *LI(o, site) = 0;
        o->num_void--;
    } else {
        o->voids[ind] = o->voids[o->num_void];
        int st[3];
        cp3(st, o->voids[o->num_void].xyz);
        *LI(o, st) = ind;
        memset(&o->voids[o->num_void], 0, sizeof(blk_t));
        *LI(o, site) = 0;
        o->num_void--;
    }
}

/* ============ rate tables ============ */
static const double KB = 0.00008617330350;   /* Get_Prob.f:70 */

/* InterpProbFromField, MS/mcevent/InterpProbFromField.f:22-57: the table
 * row at temperature t if there is one (FINDLOC), else the rows around it
 * (MINLOC of the positive differences and the row before) with integer
 * weights |T_upper - t| for the lower row and |T_lower - t| for the upper.
 * The reference copies whole interpolated tables on every call; the oracle
 * keeps the row pair and weights and mixes the entries Get_Prob reads (the
 * same values). */
static void st_interp(ora_t *o, int t)
{
    for (int i = 0; i < o->st_n; i++)
        if (o->st_T[i] == t) {
            o->st_lo = o->st_hi = i;
            return;
        }
    int iu = -1;
    for (int i = 0; i < o->st_n; i++) {
        int d = o->st_T[i] - t;
        if (d > 0 && (iu < 0 || d < o->st_T[iu] - t)) iu = i;
    }
    if (iu <= 0) ora_fail(o, "temperature %d K outside the probability table", t);
    o->st_lo = iu - 1;
    o->st_hi = iu;
    o->st_wl = abs(o->st_T[iu] - t);
    o->st_wu = abs(o->st_T[iu - 1] - t);
}
static double st_mix(const ora_t *o, double lo, double hi)
{
    if (o->st_lo == o->st_hi) return lo;
    return ((double)o->st_wl * lo + (double)o->st_wu * hi) / (double)(o->st_wl + o->st_wu);
}
static int st_live(const ora_t *o) { return o->st && !o->st_fixed; }

/* PE(...) entry; the LA law of Get_Prob.f:127-149 is evaluated per element,
 * which equals recomputing the whole table and reading one entry. */
static double pe_entry(ora_t *o, int s, int i1, int i2, int i3, int i4, int i5, int i6, int temperature)
{
    if (st_live(o))
        return st_mix(o, o->st_E[o->st_lo][s - 1][i1][i2][i3][i4][i5][i6], o->st_E[o->st_hi][s - 1][i1][i2][i3][i4][i5][i6]);
    double v = o->ptransE[s - 1][i1][i2][i3][i4][i5][i6];
    if (o->la2) return v != 0.0 ? o->lap.P0[s - 1] * exp(-v / (KB * (double)temperature)) : 0.0;
    if (o->init_st[0] == 'L' && o->init_st[1] == 'A') {
        double e = o->P0 * exp(-v / (KB * (double)temperature));
        return e * (v != 0.0 ? 1.0 : 0.0);
    }
    return v;
}
static double la2_pd(ora_t *o, int s, int coor, int temperature);
static double pd_entry(ora_t *o, int s, int coor, int temperature)
{
    if (st_live(o)) return st_mix(o, o->st_D[o->st_lo][s - 1][coor - 1], o->st_D[o->st_hi][s - 1][coor - 1]);
    double v = o->ptransD[s - 1][coor - 1];
    if (o->la2) return la2_pd(o, s, coor, temperature);
    if (o->init_st[0] == 'L' && o->init_st[1] == 'A') {
        double e = 0.5 * o->P0 * exp(-v / (KB * o->Tm)) *
                   (1.0 + erf(((double)temperature - o->Tflex) / o->sigma));
        return e * (v != 0.0 ? 1.0 : 0.0);
    }
    return v;
}

/* Prescribed temperature of grid layer z in the current window (integer K):
 * T = Tb + Ta exp(-((t_mid - t0)/w)^2) exp(-depth/L), depth = max(0, (zsurf
 * - z) sf / 10) nm, t_mid the window midpoint.  Replaces the per-site
 * temperature bits of the LaserAnnealing variant (LA/mcevent/Get_Prob.f:131). */
static int la2_temp(ora_t *o, int z)
{
    const ora_la_t *p = &o->lap;
    double tmid = ((double)o->la_win + 0.5) * p->tau;
    double g = (tmid - p->t0) / p->w;
    double depth = (p->zsurf - (double)z) * o->sf * 0.1;
    if (depth < 0.0) depth = 0.0;
    return (int)rint(p->Tb + p->Ta * exp(-g * g) * exp(-depth / p->L_nm));
}

/* Solidification of species s on a liquid site of coordination coor,
 * LaserAnnealing mcevent/Get_Prob.f:147-151 (liquid fraction xliq). */
static double la2_pd(ora_t *o, int s, int coor, int temperature)
{
    double v = o->ptransD[s - 1][coor - 1];
    /* empty sites above the initial surface are vacuum, not liquid */
    if (v == 0.0 || !(o->xliq[s - 1] > 0.0) || (double)o->la_cur_z > o->lap.zsurf) return 0.0;
    return 0.5 * o->lap.P0[s - 1] * o->xliq[s - 1] * exp(-v / (KB * o->lap.Tm[s - 1])) *
           (1.0 + erf(((double)temperature - o->lap.Tflex[s - 1]) / o->lap.sigma[s - 1]));
}

/* IndexEvent_Abs, MS/mcevent/Get_Prob.f:22-52 */
static int index_event_abs(ora_t *o, int coor, double ptmp, double pdepo)
{
    int res = 0;
    if (o->ncov == 1) return 6;
    for (int i = 1; i <= o->ncov; i++) {
        double pmin, pmax, s = 0.0;
        if (i == 1) {
            pmin = pdepo;
            pmax = pdepo + o->ptransAbs[0][coor];
        } else {
            for (int k = 0; k < i - 1; k++) s += o->ptransAbs[k][coor];
            pmin = pdepo + s;
            s = 0.0;
            for (int k = 0; k < i; k++) s += o->ptransAbs[k][coor];
            pmax = pdepo + s;
        }
        if (ptmp > pmin && ptmp <= pmax) res = 5 + i;
    }
    return res;
}

static double sum_abs(ora_t *o, int coor)
{   /* SUM(PtransAbs(:,Coor)) over NCovMax entries */
    double s = 0.0;
    for (int k = 0; k < NCOV_MAX; k++) s += o->ptransAbs[k][coor];
    return s;
}

static void get_nn_list(ora_t *o, int ind, int which, int out[4][3])
{
    if (which == 1) memcpy(out, o->mc[ind].nn, sizeof(int) * 12);
    else memcpy(out, o->bulk[ind].nn, sizeof(int) * 12);
}

static int in_list(int nn[4][3], const int site[3])
{
    int r = 0;
    for (int j = 0; j < 4; j++)
        if (same3(nn[j], site)) r = 1;
    return r;
}

/* Get_Prob, MS/mcevent/Get_Prob.f:54-331 */
static void get_prob(ora_t *o, int occ, int nsic, int covind, int coor,
                     const int site[3], int nextn[4][3], int *index_event, double *prob_event)
{
    int temperature = 0;
    int la = (o->init_st[0] == 'L' && o->init_st[1] == 'A');
    if (o->la2) {
        temperature = la2_temp(o, site[2]);
        o->la_cur_z = site[2];
    } else if (la) {
        temperature = ibits(*LC(o, site), POS_T, LEN_T);
        if (temperature == 0) ora_fail(o, "Temperature is zero in get_prob()");
    } else if (st_live(o)) {                   /* Get_Prob.f:77-91 */
        temperature = ibits(*LC(o, site), POS_T, LEN_T);
        if (temperature == 0) ora_fail(o, "Temperature is zero in get_prob()");
        st_interp(o, temperature);
    }
    if (covind > 0 && covind < WALL) {            /* desorption, :91-119 */
        if (occ != 0) ora_fail(o, "ERROR Covind!=0 with Occ!=0 in get_prob");
        if (coor <= 3) {
            *index_event = 5;
            int icov = 0;
            for (int j = 1; j <= o->ncov; j++)
                if (o->list_cov[j - 1] == covind) { icov = j; break; }
            if (icov == 0) ora_fail(o, "ERROR: could not find CovInd=%d inside ListCov", covind);
            *prob_event = o->ptransDes[icov - 1][coor];
        } else {
            *index_event = 0;
            *prob_event = 0.0;
            if (coor > 4) lg(o, " anomalous coordination in desorption\n");
        }
    } else if (occ == 0) {                       /* :154-214 */
        if (coor == 1) {
            int coornn = ibits(*LC(o, nextn[0]), POS_COOR, LEN_COOR);
            if (coornn >= 2) {
                double pd1 = pd_entry(o, 1, coor, temperature);
                double pd2 = pd_entry(o, 2, coor, temperature);
                double pd3 = pd_entry(o, 3, coor, temperature);
                double pdep = pd1 + pd2 + pd3;
                double pabs = sum_abs(o, coor);
                double ptot = pdep + pabs;
                double pcurr = rnd(o) * ptot;
                if (pcurr <= pdep) {
                    if (pcurr <= pd1) *index_event = 1;
                    else if (pcurr > pd1 + pd2) *index_event = 3;
                    else *index_event = 2;
                } else {
                    *index_event = index_event_abs(o, coor, pcurr, pdep);
                }
                *prob_event = ptot;
            } else {
                *index_event = 1;
                *prob_event = (double)1.e-8f;
            }
        } else if (coor == 2 || coor == 3) {
            double pd1 = pd_entry(o, 1, coor, temperature);
            double pd2 = pd_entry(o, 2, coor, temperature);
            double pd3 = pd_entry(o, 3, coor, temperature);
            double pdep = pd1 + pd2 + pd3;
            double pabs = sum_abs(o, coor);
            double ptot = pdep + pabs;
            double pcurr = rnd(o) * ptot;
            if (pcurr <= pdep) {
                if (pcurr <= pd1) *index_event = 1;
                else if (pcurr > pd1 + pd2) *index_event = 3;
                else *index_event = 2;
            } else {
                *index_event = index_event_abs(o, coor, pcurr, pdep);
            }
            *prob_event = ptot;
        } else if (coor >= 4) {
            *index_event = 0;
            *prob_event = 0.0;
            if (coor > 4) lg(o, " anomalous coordination\n");
        } else {
            lg(o, " anomalous coordination %d\n", coor);
        }
    } else {                                      /* occupied, :215-323 */
        int n_si = 0, n_c = 0, n_b = 0, n_wall = 0;
        int covnn[NCOV_MAX] = {0, 0, 0};
        for (int i = 0; i < 4; i++) {
            int32_t v = *LC(o, nextn[i]);
            int occn = ibits(v, POS_OCC, LEN_OCC);
            int covindn = ibits(v, POS_INDEX, LEN_INDEX);
            int coornn = ibits(v, POS_COOR, LEN_COOR);
            if (occn != 0) {
                if (covindn != WALL) {
                    int indnn = *LI(o, nextn[i]);
                    int nnn[4][3];
                    get_nn_list(o, indnn, (coornn >= 1 && coornn <= 3) ? 1 : 2, nnn);
                    if (in_list(nnn, site)) {
                        int sioc = ibits(v, POS_SIC, LEN_SIC);
                        if (sioc == 1) n_si++;
                        if (sioc == 2) n_c++;
                        if (sioc == 3) n_b++;
                    }
                } else {
                    n_wall++;
                }
            } else if (covindn != 0) {
                int indnn = *LI(o, nextn[i]);
                int nnn[4][3];
                get_nn_list(o, indnn, 1, nnn);
                if (in_list(nnn, site)) {
                    int icov = 0;
                    for (int j = 1; j <= o->ncov; j++)
                        if (o->list_cov[j - 1] == covindn) { icov = j; break; }
                    if (icov == 0) ora_fail(o, "ERROR: could not find CovIndN=%d inside ListCov", covindn);
                    covnn[icov - 1]++;
                }
            }
        }
        int tot = n_si + n_c + n_b + n_wall;
        if (tot != coor)
            ora_fail(o, "Get Prob Error N_Si+N_C+N_B+N_wall.NE.Coor at %d %d %d (coor %d, census %d)",
                     site[0], site[1], site[2], coor, tot);
        if (tot > 3) {
            *index_event = 0;
            *prob_event = 0.0;
        } else if (tot == 0) {
            *index_event = 4;
            *prob_event = 100000.0 * o->tree[1];
        } else {
            *index_event = 4;
            int c1 = 0, c2 = 0, c3 = 0;
            if (o->ncov >= 1) c1 = covnn[0];
            if (o->ncov >= 2) c2 = covnn[1];
            if (o->ncov >= 3) c3 = covnn[2];
            *prob_event = pe_entry(o, nsic, n_si + n_wall, n_c, n_b, c1, c2, c3, temperature);
        }
    }
    /* LA2: a liquid-starved site keeps its list entry (the selection of
     * ora_la_run_until recomputes every rate) */
    if (o->la2 && *index_event != 0 && *prob_event == 0.0) *prob_event = 1e-300;
    if (*index_event != 0 && *prob_event < (double)1e-12f && !o->la2)
        lg(o, " %d %.17g %d\n", *index_event, *prob_event, coor);
}

/* ============ geometry: MS/lattice/FIND_SN.f, FIND_NN.f ============ */
static int isign_f(int a, int b) { int m = abs(a); return b >= 0 ? m : -m; }

/* FIND_SN, MS/lattice/FIND_SN.f:26-84 */
static void find_sn(const int site[3], const int sitec_in[3], int sn_in[4][3],
                    int zig[3][3], int arm[3][3], int lx, int ly)
{
    int sn[3][3], sitec[3];
    for (int i = 0; i < 3; i++) cp3(sn[i], sn_in[i]);
    cp3(sitec, sitec_in);
    if (abs(site[0] - sitec[0]) > lx / 2) sitec[0] += isign_f(lx, site[0] - sitec[0]);
    if (abs(site[1] - sitec[1]) > ly / 2) sitec[1] += isign_f(ly, site[1] - sitec[1]);
    for (int i = 0; i < 3; i++) {
        if (abs(site[0] - sn[i][0]) > lx / 2) sn[i][0] += isign_f(lx, site[0] - sn[i][0]);
        if (abs(site[1] - sn[i][1]) > ly / 2) sn[i][1] += isign_f(ly, site[1] - sn[i][1]);
    }
    double cent[3], ax[3];
    for (int k = 0; k < 3; k++) {
        cent[k] = 0.5 * ((double)sitec[k] + (double)(float)site[k]);
        ax[k] = (double)site[k] - (double)sitec[k];
    }
    double snorm = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    for (int k = 0; k < 3; k++) ax[k] = ax[k] / snorm;
    const double shift = (double)8.6602254037f;
    for (int i = 0; i < 3; i++) {
        for (int k = 0; k < 3; k++) {
            double rz = 2.0 * cent[k] - (double)sn[i][k];
            double ra = (double)sn[i][k] + shift * ax[k];
            zig[i][k] = (int)lround(rz);
            arm[i][k] = (int)lround(ra);
        }
        if (zig[i][0] >= lx) zig[i][0] -= lx;
        if (zig[i][0] < 0) zig[i][0] += lx;
        if (zig[i][1] >= ly) zig[i][1] -= ly;
        if (zig[i][1] < 0) zig[i][1] += ly;
        if (arm[i][0] >= lx) arm[i][0] -= lx;
        if (arm[i][0] < 0) arm[i][0] += lx;
        if (arm[i][1] >= ly) arm[i][1] -= ly;
        if (arm[i][1] < 0) arm[i][1] += ly;
    }
}

/* FIND_NN, MS/lattice/FIND_NN.f:25-77 */
static void find_nn(const int site1[3], const int site2[3], const int sitec[3],
                    int newsite[2][3], int lx, int ly)
{
    const double pi = (double)3.14159265358979323f;
    int s11[3], s22[3];
    cp3(s11, site1);
    cp3(s22, site2);
    if (abs(sitec[0] - s11[0]) > lx / 2) s11[0] += isign_f(lx, sitec[0] - s11[0]);
    if (abs(sitec[1] - s11[1]) > ly / 2) s11[1] += isign_f(ly, sitec[1] - s11[1]);
    if (abs(sitec[0] - s22[0]) > lx / 2) s22[0] += isign_f(lx, sitec[0] - s22[0]);
    if (abs(sitec[1] - s22[1]) > ly / 2) s22[1] += isign_f(ly, sitec[1] - s22[1]);
    double ax[3];
    for (int k = 0; k < 3; k++) ax[k] = (double)sitec[k] - (double)s11[k];
    double snorm = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    for (int k = 0; k < 3; k++) ax[k] = ax[k] / snorm;
    for (int irot = 1; irot <= 2; irot++) {
        double cth = cos((double)(2 * irot) * pi / 3.0);
        double sth = sin((double)(2 * irot) * pi / 3.0);
        double rot[3][3];   /* rot[i][j] = Rot(i+1,j+1) */
        for (int i = 0; i < 3; i++) rot[i][i] = ax[i] * ax[i] * (1.0 - cth) + cth;
        rot[1][0] = ax[0] * ax[1] * (1.0 - cth) - ax[2] * sth;
        rot[0][1] = ax[0] * ax[1] * (1.0 - cth) + ax[2] * sth;
        rot[2][0] = ax[0] * ax[2] * (1.0 - cth) + ax[1] * sth;
        rot[0][2] = ax[0] * ax[2] * (1.0 - cth) - ax[1] * sth;
        rot[2][1] = ax[1] * ax[2] * (1.0 - cth) - ax[0] * sth;
        rot[1][2] = ax[1] * ax[2] * (1.0 - cth) + ax[0] * sth;
        for (int k = 0; k < 3; k++) {
            double r = 0.0;
            for (int l = 0; l < 3; l++)
                r = r + rot[l][k] * ((double)s22[l] - (double)sitec[l]);
            newsite[irot - 1][k] = (int)lround(r) + sitec[k];
        }
        int *ns = newsite[irot - 1];
        if (ns[0] >= lx) ns[0] -= lx;
        if (ns[0] < 0) ns[0] += lx;
        if (ns[1] >= ly) ns[1] -= ly;
        if (ns[1] < 0) ns[1] += ly;
    }
}

/* IF_Arm_Choice, MS/mcevent/IF_Arm_Choice.f:21-56 */
static int if_arm_choice(ora_t *o, int zig[3][3], int arm[3][3])
{
    int ca = 0, cz = 0;
    for (int i = 0; i < 3; i++) {
        ca += ibits(*LC(o, arm[i]), POS_COOR, LEN_COOR);
        cz += ibits(*LC(o, zig[i]), POS_COOR, LEN_COOR);
    }
    if (cz > ca) return 0;
    if (cz == ca) return (rnd(o) <= o->ptrans_zig) ? 0 : 1;
    return 1;
}

/* ============ events ============ */
/* Deposition, MS/mcevent/deposition.f:24-251 */
static void deposition(ora_t *o, int indvoid, int iatom)
{
    int site[3], nextn[4][3], nextnn[4][3], nextnnn[4][3];
    int index_event;
    double prob;
    cp3(site, o->mc[indvoid].xyz);
    int32_t *ls = LC(o, site);
    int coor = ibits(*ls, POS_COOR, LEN_COOR);
    int coor_old = coor;
    mvbits(1, LEN_OCC, ls, POS_OCC);
    mvbits(iatom, LEN_SIC, ls, POS_SIC);
    o->cur_arm = 0;
    if (coor == 1) {                              /* :49-74 */
        int sitec[3];
        cp3(sitec, o->mc[indvoid].nn[0]);
        int indnn = *LI(o, sitec);
        int snsite[4][3];
        memset(snsite, 0, sizeof snsite);
        int j = 0;
        for (int i = 0; i < 4; i++) {
            if (!same3(o->mc[indnn].nn[i], site)) {
                if (j < 4) cp3(snsite[j], o->mc[indnn].nn[i]);
                j++;
            }
        }
        int zig[3][3], arm[3][3];
        find_sn(site, sitec, snsite, zig, arm, o->lx, o->ly);
        int if_arm = if_arm_choice(o, zig, arm);
        o->cur_arm = if_arm;
        for (int i = 0; i < 3; i++) cp3(o->mc[indvoid].nn[i + 1], if_arm ? arm[i] : zig[i]);
    }
    memcpy(nextn, o->mc[indvoid].nn, sizeof nextn);
    for (int i = 0; i < 4; i++) {                 /* :78-235 */
        int32_t *ln = LC(o, nextn[i]);
        int occ = ibits(*ln, POS_OCC, LEN_OCC);
        int indnn = *LI(o, nextn[i]);
        int coornn = ibits(*ln, POS_COOR, LEN_COOR);
        int covind = ibits(*ln, POS_INDEX, LEN_INDEX);
        memset(nextnn, 0, sizeof nextnn);
        if (occ == 0) {
            if (coornn == 0) {
                coornn = 1;
                mvbits(coornn, LEN_COOR, ln, POS_COOR);
                cp3(nextnn[0], site);
                get_prob(o, 0, 0, covind, coornn, nextn[i], nextnn, &index_event, &prob);
                if (index_event != 0) add_mc(o, nextn[i], nextnn, index_event, prob);
            } else if (coornn == 1) {
                memcpy(nextnn, o->mc[indnn].nn, sizeof nextnn);
                int dx = abs(nextnn[0][0] - site[0]);
                if (o->lx - dx < dx) dx = o->lx - dx;
                int dy = abs(nextnn[0][1] - site[1]);
                if (o->ly - dy < dy) dy = o->ly - dy;
                int dz = nextnn[0][2] - site[2];
                int dis = dx * dx + dy * dy + dz * dz;
                if (dis == 72) {
                    coornn = 2;
                    cp3(nextnn[1], site);
                    int newsite[2][3];
                    find_nn(nextnn[0], nextnn[1], nextn[i], newsite, o->lx, o->ly);
                    for (int j = 2; j < 4; j++) {
                        cp3(nextnn[j], newsite[j - 2]);
                        int32_t v = *LC(o, nextnn[j]);
                        int occn = ibits(v, POS_OCC, LEN_OCC);
                        if (occn != 0) {
                            int coornnn = ibits(v, POS_COOR, LEN_COOR);
                            int covindnnn = ibits(v, POS_INDEX, LEN_INDEX);
                            if (coornnn <= 3 && covindnnn != WALL) {
                                int indnnn = *LI(o, nextnn[j]);
                                memcpy(nextnnn, o->mc[indnnn].nn, sizeof nextnnn);
                                if (in_list(nextnnn, nextn[i])) coornn++;
                            }
                        }
                    }
                    mvbits(coornn, LEN_COOR, ln, POS_COOR);
                    memcpy(o->mc[indnn].nn, nextnn, sizeof nextnn);
                    get_prob(o, 0, 0, covind, coornn, nextn[i], nextnn, &index_event, &prob);
                    if (index_event == 0) {
                        erase_mc(o, nextn[i]);
                        add_void(o, nextn[i], nextnn);
                    } else {
                        o->mc[indnn].ind_event = index_event;
                        o->mc[indnn].prob = prob;
                        update_tree(o, indnn, prob);
                    }
                }
            } else if (coornn == 2 || coornn == 3) {
                memcpy(nextnn, o->mc[indnn].nn, sizeof nextnn);
                if (in_list(nextnn, site)) {
                    coornn++;
                    mvbits(coornn, LEN_COOR, ln, POS_COOR);
                    get_prob(o, 0, 0, covind, coornn, nextn[i], nextnn, &index_event, &prob);
                    if (index_event == 0) {
                        erase_mc(o, nextn[i]);
                        add_void(o, nextn[i], nextnn);
                    } else {
                        o->mc[indnn].ind_event = index_event;
                        o->mc[indnn].prob = prob;
                        update_tree(o, indnn, prob);
                    }
                }
            }
        } else {
            if (covind != WALL) {
                if (covind != 0) ora_fail(o, "ERROR in deposition: Site can only have NN with CovInd=0 or 113 when its Occ=1");
                if (coornn <= 3) {
                    memcpy(nextnn, o->mc[indnn].nn, sizeof nextnn);
                    if (in_list(nextnn, site)) {
                        coornn++;
                        mvbits(coornn, LEN_COOR, ln, POS_COOR);
                        int sioc = ibits(*ln, POS_SIC, LEN_SIC);
                        get_prob(o, 1, sioc, covind, coornn, nextn[i], nextnn, &index_event, &prob);
                        if (index_event == 0) {
                            erase_mc(o, nextn[i]);
                            add_bulk(o, nextn[i], nextnn);
                        } else {
                            o->mc[indnn].ind_event = index_event;
                            o->mc[indnn].prob = prob;
                            update_tree(o, indnn, prob);
                        }
                        if (coor_old == 1 && i >= 1) coor++;
                    }
                }
            } else {
                coor++;
            }
        }
    }
    indvoid = *LI(o, site);                       /* :236-250 */
    if (coor != coor_old) mvbits(coor, LEN_COOR, ls, POS_COOR);
    get_prob(o, 1, iatom, 0, coor, site, nextn, &index_event, &prob);
    if (index_event == 0) {
        erase_mc(o, site);
        add_bulk(o, site, nextn);
    } else {
        o->mc[indvoid].ind_event = index_event;
        o->mc[indvoid].prob = prob;
        update_tree(o, indvoid, prob);
    }
}

/* Evaporation, MS/mcevent/Evaporation.f:25-262 */
static void evaporation(ora_t *o, int indatom)
{
    int site[3], nextn[4][3], nextnn[4][3], nextnnn[4][3];
    int index_event;
    double prob;
    int la_or_st = (o->init_st[0] == 'L' && o->init_st[1] == 'A') ||
                   (o->init_st[0] == 'S' && o->init_st[1] == 'T');
    cp3(site, o->mc[indatom].xyz);
    int32_t *ls = LC(o, site);
    int iatom = ibits(*ls, POS_SIC, LEN_SIC);
    if (iatom >= 1 && iatom <= NCRYSTAL_MAX) o->count_crystal[iatom - 1]--;
    int coor = ibits(*ls, POS_COOR, LEN_COOR);
    mvbits(0, LEN_OCC, ls, POS_OCC);
    mvbits(0, LEN_SIC, ls, POS_SIC);
    memcpy(nextn, o->mc[indatom].nn, sizeof nextn);
    for (int i = 0; i < 4; i++) {
        int32_t *ln = LC(o, nextn[i]);
        int occ = ibits(*ln, POS_OCC, LEN_OCC);
        int coornn = ibits(*ln, POS_COOR, LEN_COOR);
        int indnn = *LI(o, nextn[i]);
        int covind = ibits(*ln, POS_INDEX, LEN_INDEX);
        memset(nextnn, 0, sizeof nextnn);
        if (occ == 0) {
            if (coornn == 1) {                    /* :51-68 */
                memcpy(nextnn, o->mc[indnn].nn, sizeof nextnn);
                if (in_list(nextnn, site)) {
                    erase_mc(o, nextn[i]);
                    if (la_or_st) {
                        int t = ibits(*ln, POS_T, LEN_T);
                        *ln = 0;
                        mvbits(t, LEN_T, ln, POS_T);
                    } else {
                        *ln = 0;
                    }
                }
            } else if (coornn == 2) {             /* :69-123 */
                memcpy(nextnn, o->mc[indnn].nn, sizeof nextnn);
                if (in_list(nextnn, site)) {
                    coornn = 1;
                    mvbits(coornn, LEN_COOR, ln, POS_COOR);
                    for (int j = 0; j < 4; j++) {
                        int32_t v = *LC(o, nextnn[j]);
                        int occn = ibits(v, POS_OCC, LEN_OCC);
                        if (occn == 0) {
                            memset(o->mc[indnn].nn[j], 0, sizeof(int) * 3);
                        } else {
                            int coornnn = ibits(v, POS_COOR, LEN_COOR);
                            int covindnn = ibits(v, POS_INDEX, LEN_INDEX);
                            if (coornnn <= 3 && covindnn != WALL) {
                                int indnnn = *LI(o, nextnn[j]);
                                memcpy(nextnnn, o->mc[indnnn].nn, sizeof nextnnn);
                                if (in_list(nextnnn, nextn[i]))
                                    cp3(o->nbuff, o->mc[indnn].nn[j]);
                            }
                            memset(o->mc[indnn].nn[j], 0, sizeof(int) * 3);
                        }
                    }
                    cp3(o->mc[indnn].nn[0], o->nbuff);
                    get_prob(o, 0, 0, covind, coornn, nextn[i], nextnn, &index_event, &prob);
                    o->mc[indnn].ind_event = index_event;
                    o->mc[indnn].prob = prob;
                    update_tree(o, indnn, prob);
                }
            } else if (coornn == 3) {             /* :124-141 */
                memcpy(nextnn, o->mc[indnn].nn, sizeof nextnn);
                if (in_list(nextnn, site)) {
                    coornn = 2;
                    mvbits(coornn, LEN_COOR, ln, POS_COOR);
                    get_prob(o, 0, 0, covind, coornn, nextn[i], nextnn, &index_event, &prob);
                    o->mc[indnn].ind_event = index_event;
                    o->mc[indnn].prob = prob;
                    update_tree(o, indnn, prob);
                }
            } else if (coornn == 4) {             /* :142-164 */
                memcpy(nextnn, o->voids[indnn].nn, sizeof nextnn);
                if (in_list(nextnn, site)) {
                    coornn = 3;
                    mvbits(coornn, LEN_COOR, ln, POS_COOR);
                    get_prob(o, 0, 0, covind, coornn, nextn[i], nextnn, &index_event, &prob);
                    erase_void(o, nextn[i]);
                    add_mc(o, nextn[i], nextnn, index_event, prob);
                }
            }
        } else {
            if (covind != WALL) {                 /* :166-210 */
                if (covind != 0) ora_fail(o, "ERROR in evaporation: NN with CovInd not 0/113 and Occ=1");
                if (coornn == 4) {
                    memcpy(nextnn, o->bulk[indnn].nn, sizeof nextnn);
                    if (in_list(nextnn, site)) {
                        coornn = 3;
                        mvbits(coornn, LEN_COOR, ln, POS_COOR);
                        int sioc = ibits(*ln, POS_SIC, LEN_SIC);
                        get_prob(o, 1, sioc, covind, coornn, nextn[i], nextnn, &index_event, &prob);
                        erase_bulk(o, nextn[i]);
                        add_mc(o, nextn[i], nextnn, index_event, prob);
                    }
                } else {
                    memcpy(nextnn, o->mc[indnn].nn, sizeof nextnn);
                    if (in_list(nextnn, site)) {
                        coornn--;
                        mvbits(coornn, LEN_COOR, ln, POS_COOR);
                        int sioc = ibits(*ln, POS_SIC, LEN_SIC);
                        get_prob(o, 1, sioc, covind, coornn, nextn[i], nextnn, &index_event, &prob);
                        o->mc[indnn].ind_event = index_event;
                        o->mc[indnn].prob = prob;
                        update_tree(o, indnn, prob);
                    }
                }
            } else {
                coor--;
            }
        }
    }
    indatom = *LI(o, site);                       /* :216-261 */
    mvbits(coor, LEN_COOR, ls, POS_COOR);
    if (coor == 0) {
        erase_mc(o, site);
    } else {
        get_prob(o, 0, 0, 0, coor, site, nextn, &index_event, &prob);
        o->mc[indatom].ind_event = index_event;
        o->mc[indatom].prob = prob;
        if (coor == 1) {
            memcpy(nextn, o->mc[indatom].nn, sizeof nextn);
            for (int i = 0; i < 4; i++) {
                int32_t v = *LC(o, nextn[i]);
                int occn = ibits(v, POS_OCC, LEN_OCC);
                if (occn == 0) {
                    memset(o->mc[indatom].nn[i], 0, sizeof(int) * 3);
                } else {
                    int coornn = ibits(v, POS_COOR, LEN_COOR);
                    int covindnn = ibits(v, POS_INDEX, LEN_INDEX);
                    if (coornn <= 3 && covindnn != WALL) {
                        int indnn = *LI(o, nextn[i]);
                        memcpy(nextnn, o->mc[indnn].nn, sizeof nextnn);
                        if (in_list(nextnn, site)) cp3(o->nbuff, o->mc[indatom].nn[i]);
                    }
                    memset(o->mc[indatom].nn[i], 0, sizeof(int) * 3);
                }
            }
            cp3(o->mc[indatom].nn[0], o->nbuff);
        }
        update_tree(o, indatom, prob);
    }
}

/* absorption, MS/mcevent/absorption.f:25-78 */
static void absorption(ora_t *o, int indvoid, int covind)
{
    int site[3], nextn[4][3], nextnn[4][3], index_event;
    double prob;
    cp3(site, o->mc[indvoid].xyz);
    int32_t *ls = LC(o, site);
    int coor = ibits(*ls, POS_COOR, LEN_COOR);
    mvbits(covind, LEN_INDEX, ls, POS_INDEX);
    memcpy(nextn, o->mc[indvoid].nn, sizeof nextn);
    for (int i = 0; i < 4; i++) {
        int32_t v = *LC(o, nextn[i]);
        int occn = ibits(v, POS_OCC, LEN_OCC);
        int indnn = *LI(o, nextn[i]);
        int coorn = ibits(v, POS_COOR, LEN_COOR);
        if (occn != 0) {
            int covindn = ibits(v, POS_INDEX, LEN_INDEX);
            if (covindn != WALL && coorn <= 3) {
                memcpy(nextnn, o->mc[indnn].nn, sizeof nextnn);
                if (in_list(nextnn, site)) {
                    int sioc = ibits(v, POS_SIC, LEN_SIC);
                    get_prob(o, 1, sioc, covindn, coorn, nextn[i], nextnn, &index_event, &prob);
                    o->mc[indnn].ind_event = index_event;
                    o->mc[indnn].prob = prob;
                    update_tree(o, indnn, prob);
                }
            }
        }
    }
    get_prob(o, 0, 0, covind, coor, site, nextn, &index_event, &prob);
    o->mc[indvoid].ind_event = index_event;
    o->mc[indvoid].prob = prob;
    update_tree(o, indvoid, prob);
}

/* desorption, MS/mcevent/desorption.f:25-117 */
static void desorption_nn(ora_t *o, const int site[3], const int nn[3])
{
    int nextnn[4][3], index_event;
    double prob;
    int32_t v = *LC(o, nn);
    int occn = ibits(v, POS_OCC, LEN_OCC);
    int indnn = *LI(o, nn);
    int coorn = ibits(v, POS_COOR, LEN_COOR);
    if (occn != 0) {
        int covindn = ibits(v, POS_INDEX, LEN_INDEX);
        if (covindn != WALL) {
            memcpy(nextnn, o->mc[indnn].nn, sizeof nextnn);
            if (in_list(nextnn, site)) {
                int sioc = ibits(v, POS_SIC, LEN_SIC);
                get_prob(o, 1, sioc, covindn, coorn, nn, nextnn, &index_event, &prob);
                o->mc[indnn].ind_event = index_event;
                o->mc[indnn].prob = prob;
                update_tree(o, indnn, prob);
            }
        }
    }
}

static void desorption(ora_t *o, int indatom)
{
    int site[3], nextn[4][3], index_event;
    double prob;
    cp3(site, o->mc[indatom].xyz);
    int32_t *ls = LC(o, site);
    int covind = ibits(*ls, POS_INDEX, LEN_INDEX);
    if (covind == o->list_cov[0]) o->count_cov[0]--;
    else if (covind == o->list_cov[1]) o->count_cov[1]--;
    else if (covind == o->list_cov[2]) o->count_cov[2]--;
    int coor = ibits(*ls, POS_COOR, LEN_COOR);
    mvbits(0, LEN_INDEX, ls, POS_INDEX);
    memcpy(nextn, o->mc[indatom].nn, sizeof nextn);
    if (coor == 1) {
        desorption_nn(o, site, nextn[0]);
    } else {
        for (int i = 0; i < 4; i++) desorption_nn(o, site, nextn[i]);
    }
    get_prob(o, 0, 0, 0, coor, site, nextn, &index_event, &prob);
    o->mc[indatom].ind_event = index_event;
    o->mc[indatom].prob = prob;
    update_tree(o, indatom, prob);
}

/* ============ initial structures ============ */
static void std_neighbours(ora_t *o, const int site[3], int first, int nextn[4][3])
{
    for (int i = 0; i < 4; i++) {
        for (int k = 0; k < 3; k++) nextn[i][k] = site[k] + JUMPDIA[first + i][k];
        if (nextn[i][0] >= o->lx) nextn[i][0] -= o->lx;
        if (nextn[i][0] < 0) nextn[i][0] += o->lx;
        if (nextn[i][1] >= o->ly) nextn[i][1] -= o->ly;
        if (nextn[i][1] < 0) nextn[i][1] += o->ly;
    }
}

/* diamond site test used by every initializer (e.g. SetSi.f:52-57):
 * returns 0 (not a site), 1 ((x1+y1+z1) mod 4 == 0), 2 (== 3) */
static int dia_kind(int x, int y, int z)
{
    if (x % 3 || y % 3 || z % 3) return 0;
    int x1 = x / 3, y1 = y / 3, z1 = z / 3;
    if ((x1 % 2) != (y1 % 2) || (x1 % 2) != (z1 % 2)) return 0;
    int m = (x1 + y1 + z1) % 4;
    if (m == 0) return 1;
    if (m == 3) return 2;
    return 0;
}

static void set_walls(ora_t *o, int z0, int z1)
{
    for (int z = z0; z <= z1; z++)
        for (int y = 0; y < o->ly; y++)
            for (int x = 0; x < o->lx; x++) {
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                *v = (int32_t)((uint32_t)*v | (1u << POS_OCC));
                mvbits(WALL, LEN_INDEX, v, POS_INDEX);
            }
}

/* SetSi (InitSt 'FS'), MS/initial/SetSi.f:25-221; SetSiC3C (InitSt 'F'),
 * MS/initial/SetSiC3C.f:25-199.  They differ in the walls (SetSi only),
 * the bulk start (z=6 vs z=0) and the species of the second sublattice
 * (Si vs C) and of the surface layer's rate (PtransE(1|2,2,...)). */
static void set_flat(ora_t *o, int len, int sic, int walls)
{
    int site[3], nextn[4][3], index_event;
    double prob;
    if (walls) set_walls(o, 0, 5);
    int zb = walls ? 6 : 0;
    for (int z = zb; z <= len - 4; z++)
        for (int y = 0; y < o->ly; y++)
            for (int x = 0; x < o->lx; x++) {
                int k = dia_kind(x, y, z);
                if (!k) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                int sp = (k == 2 && sic) ? POS_C : POS_SI;
                *v = (int32_t)((uint32_t)*v | (1u << sp) | (1u << POS_OCC));
                mvbits(4, LEN_COOR, v, POS_COOR);
                site[0] = x; site[1] = y; site[2] = z;
                std_neighbours(o, site, k == 1 ? 0 : 4, nextn);
                add_bulk(o, site, nextn);
            }
    for (int z = len - 3; z <= len - 1; z++)
        for (int y = 0; y < o->ly; y++)
            for (int x = 0; x < o->lx; x++) {
                int k = dia_kind(x, y, z);
                if (!k) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                int sp = (k == 2 && sic) ? POS_C : POS_SI;
                *v = (int32_t)((uint32_t)*v | (1u << sp) | (1u << POS_OCC));
                mvbits(2, LEN_COOR, v, POS_COOR);
                site[0] = x; site[1] = y; site[2] = z;
                std_neighbours(o, site, k == 1 ? 0 : 4, nextn);
                prob = o->ptransE[(k == 2 && sic) ? 1 : 0][2][0][0][0][0][0];
                add_mc(o, site, nextn, 4, prob);
            }
    for (int y = 0; y < o->ly; y++)
        for (int x = 0; x < o->lx; x++) {
            int z = len;
            int k = dia_kind(x, y, z);
            if (!k) continue;
            int32_t *v = &o->latt[lidx(o, x, y, z)];
            mvbits(2, LEN_COOR, v, POS_COOR);
            site[0] = x; site[1] = y; site[2] = z;
            std_neighbours(o, site, k == 1 ? 0 : 4, nextn);
            get_prob(o, 0, 0, 0, 2, site, nextn, &index_event, &prob);
            add_mc(o, site, nextn, index_event, prob);
        }
    if (walls) set_walls(o, o->lz - 6, o->lz - 1);
}

/* The wall block of SetSiC3Cww (MS/initial/SetSiC3Cww.f:209-218, InitSt
 * 'Fw') and SetSiC3Cwwaperture (SetSiC3Cwwaperture.f:209-223, 'Fa'): every
 * grid point of z = Lenww..LenZ-7, or with lap >= 0 those with x below
 * INT(0.5 (LenX - lap)) or from INT(0.5 (LenX + lap)), written after the
 * lists without touching them. */
static void set_wall_block(ora_t *o, int lenww, int lap)
{
    int xa = lap >= 0 ? (int)(0.5 * (o->lx - lap)) : o->lx, xb = lap >= 0 ? (int)(0.5 * (o->lx + lap)) : o->lx;
    for (int z = lenww; z <= o->lz - 7; z++)
        for (int y = 0; y < o->ly; y++)
            for (int x = 0; x < o->lx; x++) {
                if (lap >= 0 && x >= xa && x < xb) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                *v = (int32_t)((uint32_t)*v | (1u << POS_OCC));
                mvbits(WALL, LEN_INDEX, v, POS_INDEX);
            }
}

/* Get_Prob_Ini, MS/mcevent/Get_Prob_Ini.f:23-161: init-time rate of a site
 * (no reciprocity check; walls counted by their index; dummy rate 1e-6). */
static void get_prob_ini(ora_t *o, int occ, int nsic, int coor, const int site[3], int nextn[4][3],
                         int *index_event, double *prob_event)
{
    int temperature = 0;
    if (o->init_st[0] == 'L' && o->init_st[1] == 'A') {
        temperature = ibits(*LC(o, site), POS_T, LEN_T);
        if (temperature == 0) ora_fail(o, "Temperature is zero in get_prob_ini()");
    } else if (st_live(o)) {                   /* Get_Prob_Ini.f:42-53 */
        temperature = ibits(*LC(o, site), POS_T, LEN_T);
        if (temperature == 0) ora_fail(o, "Temperature is zero in get_prob_ini()");
        st_interp(o, temperature);
    }
    *index_event = 0;
    *prob_event = 0.0;
    if (occ == 0) {
        int draw = 0;
        if (coor == 1) {
            int coornn = ibits(*LC(o, nextn[0]), POS_COOR, LEN_COOR);
            if (coornn >= 2) draw = 1;
            else { *index_event = 1; *prob_event = (double)1.e-6f; }
        } else if (coor == 2 || coor == 3) {
            draw = 1;
        } else if (coor == 4) {
            lg(o, " %d Get Prob Vacancy Generation\n", coor);
        }
        if (draw) {
            double pd1 = pd_entry(o, 1, coor, temperature), pd2 = pd_entry(o, 2, coor, temperature);
            double pd3 = pd_entry(o, 3, coor, temperature);
            double ptot = pd1 + pd2 + pd3;
            double pcurr = rnd(o) * ptot;
            if (pcurr <= pd1) *index_event = 1;
            else if (pcurr > pd1 + pd2) *index_event = 3;
            else *index_event = 2;
            *prob_event = ptot;
        }
    } else {
        int n_si = 0, n_c = 0, n_b = 0, n_cov = 0;
        for (int i = 0; i < 4; i++) {
            int32_t v = *LC(o, nextn[i]);
            if (ibits(v, POS_INDEX, LEN_INDEX) == 0) {
                int sp = ibits(v, POS_SIC, LEN_SIC);
                if (sp == 1) n_si++;
                if (sp == 2) n_c++;
                if (sp == 3) n_b++;
            } else {
                n_cov++;
            }
        }
        int tot = n_si + n_c + n_b + n_cov;
        if (tot != coor) ora_fail(o, "Get Prob Error N_Si+N_C++N_B+N_cov.NE.Coor at %d %d %d", site[0], site[1], site[2]);
        if (tot > 3) {
            *index_event = 0;
            *prob_event = 0.0;
        } else if (tot == 0) {
            *index_event = 4;
            *prob_event = 100000.0 * o->tree[1];
        } else {
            *index_event = 4;
            *prob_event = pe_entry(o, nsic, n_si + n_cov, n_c, n_b, 0, 0, 0, temperature);
        }
    }
}

/* The two passes that close the free-form initial states (SetNC.f:62-234,
 * SetNCSp.f:64-236, SetInvPOff.f:113-285, SetSiFINFET.f:120-311): over the
 * box [xa,xb] x [ya,yb] x [za,zb] every diamond site gets its coordination
 * from its occupied neighbours, occupied sites with none are removed (their
 * neighbours' counts drop by one, floored at 0); then every site with
 * coor > 0 or occupied joins the MC list (Get_Prob_Ini) or, occupied with
 * coor 4, the bulk list.  With walls != 0 (SetSiFINFET) wall sites (index
 * 113) are skipped, an empty site does not count wall neighbours, and the
 * one neighbour kept for an empty coor-1 site is never a wall. */
static inline int is_wall(int32_t v) { return ibits(v, POS_INDEX, LEN_INDEX) == WALL; }

static void coor_pass(ora_t *o, int xa, int xb, int ya, int yb, int za, int zb, int walls)
{
    int site[3], nextn[4][3];
    for (int z = za; z <= zb; z++)
        for (int y = ya; y <= yb; y++)
            for (int x = xa; x <= xb; x++) {
                int k = dia_kind(x, y, z);
                if (!k) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                if (walls && is_wall(*v)) continue;
                site[0] = x; site[1] = y; site[2] = z;
                std_neighbours(o, site, k == 1 ? 0 : 4, nextn);
                int coor = 0, occ = ibits(*v, POS_OCC, LEN_OCC);
                for (int i = 0; i < 4; i++) {
                    int32_t w = *LC(o, nextn[i]);
                    if (ibits(w, POS_OCC, LEN_OCC) > 0 && (occ || !walls || !is_wall(w))) coor++;
                }
                if (occ != 0 && coor == 0) {
                    *v = 0;
                    for (int i = 0; i < 4; i++) {
                        int32_t *w = LC(o, nextn[i]);
                        int cn = ibits(*w, POS_COOR, LEN_COOR) - 1;
                        if (cn < 0) cn = 0;
                        mvbits(cn, LEN_COOR, w, POS_COOR);
                    }
                } else {
                    mvbits(coor, LEN_COOR, v, POS_COOR);
                }
            }
}

static void list_pass(ora_t *o, int xa, int xb, int ya, int yb, int za, int zb, int walls)
{
    int site[3], nextn[4][3];
    int nbuff[3] = {0, 0, 0};
    for (int z = za; z <= zb; z++)
        for (int y = ya; y <= yb; y++)
            for (int x = xa; x <= xb; x++) {
                int k = dia_kind(x, y, z);
                if (!k) continue;
                int32_t v = o->latt[lidx(o, x, y, z)];
                if (walls && is_wall(v)) continue;
                site[0] = x; site[1] = y; site[2] = z;
                std_neighbours(o, site, k == 1 ? 0 : 4, nextn);
                int occ = ibits(v, POS_OCC, LEN_OCC), coor = ibits(v, POS_COOR, LEN_COOR);
                int index_event;
                double prob;
                if (occ == 0) {
                    if (coor == 0) continue;
                    if (coor == 1) {
                        for (int i = 0; i < 4; i++) {
                            int32_t w = *LC(o, nextn[i]);
                            if (ibits(w, POS_OCC, LEN_OCC) != 0 && !(walls && is_wall(w))) cp3(nbuff, nextn[i]);
                            nextn[i][0] = nextn[i][1] = nextn[i][2] = 0;
                        }
                        cp3(nextn[0], nbuff);
                    }
                    get_prob_ini(o, 0, 0, coor, site, nextn, &index_event, &prob);
                    add_mc(o, site, nextn, index_event, prob);
                } else if (coor <= 3) {
                    get_prob_ini(o, 1, ibits(v, POS_SIC, LEN_SIC), coor, site, nextn, &index_event, &prob);
                    add_mc(o, site, nextn, index_event, prob);
                } else {
                    add_bulk(o, site, nextn);
                }
            }
}

/* SetNC, MS/initial/SetNC.f:24-235 (InitSt 'C'): a free-standing 3C
 * parallelepiped of Len1 x Len2 x Len3 grid units centred in the box (species
 * 1 on the (x1+y1+z1) mod 4 = 0 sublattice, 2 on the other), coordinations
 * and isolated-atom removal over the box grown by 10, then the lists.  With
 * sphere != 0 it is SetNCSp (MS/initial/SetNCSp.f:24-237, InitSt 'S'): the
 * cube of side Len1 cut to the ball d^2 <= Len1^2/4 around the box centre.
 * With all_si it is SetNCSpSi (MS/initial/SetNCSpSi.f, InitSt 'SS'): the
 * same ball with Si on both sublattices. */
static void set_nc(ora_t *o, int len1, int len2, int len3, int sphere, int all_si)
{
    int lx = o->lx, ly = o->ly, lz = o->lz;
    int x0 = lx / 2 - len1 / 2, x1e = lx / 2 + len1 / 2 - 1;
    int y0 = ly / 2 - len2 / 2, y1e = ly / 2 + len2 / 2 - 1;
    int z0 = lz / 2 - len3 / 2, z1e = lz / 2 + len3 / 2 - 1;
    if (!sphere) {
        lg(o, " %d %d\n", z0, lz / 2 + len3 / 2 + 1);
        lg(o, " %d %d\n", x0, lx / 2 + len1 / 2 + 1);
    }
    for (int z = z0; z <= z1e; z++)
        for (int y = y0; y <= y1e; y++)
            for (int x = x0; x <= x1e; x++) {
                if (sphere) {
                    long d2 = (long)(x - lx / 2) * (x - lx / 2) + (long)(y - ly / 2) * (y - ly / 2) +
                              (long)(z - lz / 2) * (z - lz / 2);
                    if (d2 > (long)len1 * len1 / 4) continue;
                }
                int k = dia_kind(x, y, z);
                if (!k) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                *v = (int32_t)((uint32_t)*v | (1u << (k == 1 || all_si ? POS_SI : POS_C)) | (1u << POS_OCC));
            }
    coor_pass(o, x0 - 10, x1e + 10, y0 - 10, y1e + 10, z0 - 10, z1e + 10, 0);
    list_pass(o, x0 - 10, x1e + 10, y0 - 10, y1e + 10, z0 - 10, z1e + 10, 0);
}

/* SetInvPOff, MS/initial/SetInvPOff.f:22-286 (InitSt 'I', called with
 * (Len1, Len2), MS/main.f:245-246): a 3C substrate z = 0..20 (bulk, coor 4)
 * under a 3C layer z = 21..Len3-1 from which inverted pyramids are cut, one
 * at the box centre (Lenh = LenX/2 - 1) and quarters at the four corners:
 * a site is left empty when |x-xc| + |y-yc| - 1.10 (z - Len3) <= Len for
 * any of the five centres.  The test is evaluated in single precision, as
 * the reference's default-REAL constant 1.10 makes it.  Then the two
 * closing passes over z = 21..Len3+9 on the whole x-y plane.  The same code
 * with slope 1 in integers and the species of invp_species is SetInvPC
 * ('D'), SetInvPSi ('Z'), SetInvPwAPB ('J'), SetInvPwOnlySiorC ('K') and
 * SetInvPwOnlyCorSi ('L'), MS/main.f:247-256. */
/* The species of a site of sublattice k (1, 2) at (x, y) in the inverted
 * pyramid family: 'I' SetInvPOff (1 on sublattice 1, 2 on 2), 'Z' SetInvPSi
 * (all Si), 'D' SetInvPC (all C), 'K' SetInvPwOnlySiorC (sublattices swapped
 * outside the quadrants x < LenX/2 <= y and y < LenY/2 <= x), 'L'
 * SetInvPwOnlyCorSi (swapped inside them), 'J' SetInvPwAPB (swapped where
 * x + y > LenY): antiphase domains. */
static int invp_species(int mode, int k, int x, int y, int lx, int ly)
{
    if (mode == 'I') return k;
    if (mode == 'Z') return 1;
    if (mode == 'D') return 2;
    int r = mode == 'J' ? x + y <= ly : ((x < lx / 2 && y >= ly / 2) || (x >= lx / 2 && y < ly / 2));
    if (mode == 'L') r = !r;
    return r ? k : 3 - k;
}

static void set_invp(ora_t *o, int len, int len3, int mode)
{
    int lx = o->lx, ly = o->ly;
    int lenh = lx / 2 - 1;
    int site[3], nextn[4][3];
    lg(o, " %d %d %d\n", lenh, len, len3);
    for (int z = 0; z <= 20; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int k = dia_kind(x, y, z);
                if (!k) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                int sp = invp_species(mode, k, x, y, lx, ly);
                *v = (int32_t)((uint32_t)*v | (1u << (sp == 1 ? POS_SI : POS_C)) | (1u << POS_OCC));
                mvbits(4, LEN_COOR, v, POS_COOR);
                site[0] = x; site[1] = y; site[2] = z;
                std_neighbours(o, site, k == 1 ? 0 : 4, nextn);
                add_bulk(o, site, nextn);
            }
    const int cx[5] = {lenh, 0, lx, 0, lx}, cy[5] = {lenh, 0, 0, ly, ly};
    for (int z = 21; z <= len3 - 1; z++) {
        float dz = 1.10f * (float)(z - len3);
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int k = dia_kind(x, y, z);
                if (!k) continue;
                int pit = 0;
                for (int c = 0; c < 5 && !pit; c++) {
                    int d = abs(x - cx[c]) + abs(y - cy[c]);
                    /* slope 1.10 (a default-REAL literal) for SetInvPOff, 1 (integer) for the others */
                    pit = mode == 'I' ? (float)d - dz <= (float)len : d - (z - len3) <= len;
                }
                if (pit) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                int sp = invp_species(mode, k, x, y, lx, ly);
                *v = (int32_t)((uint32_t)*v | (1u << (sp == 1 ? POS_SI : POS_C)) | (1u << POS_OCC));
            }
    }
    coor_pass(o, 0, lx - 1, 0, ly - 1, 21, len3 + 9, 0);
    list_pass(o, 0, lx - 1, 0, ly - 1, 21, len3 + 9, 0);
}

/* SetSiFINFET, MS/initial/SetSiFINFET.f:23-312 (InitSt 'FF', Len1..Len4
 * each rounded down to a multiple of 24, MS/main.f:273-278): walls (index
 * 113) at z = 0..5 and z = LenZ-6..LenZ-1, a wall layer z = Lenwwtop..LenZ-7
 * and, from z = Lenww up, side walls leaving an aperture of Laperture grid
 * units around the box centre in x; Si (both sublattices) fills the non-wall
 * sites of z = 6..Len-1; then the two closing passes in wall mode over
 * z = 6..Lenwwtop+9. */
static void set_finfet(ora_t *o, int len, int lenww, int lenwwtop, int lap)
{
    int lx = o->lx, ly = o->ly, lz = o->lz;
    int xl = (int)(0.5f * (float)(lx - lap)), xr = (int)(0.5f * (float)(lx + lap));
    set_walls(o, 0, 5);
    for (int z = lenww; z <= lz - 7; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                if (x >= xl && x < xr) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                *v = (int32_t)((uint32_t)*v | (1u << POS_OCC));
                mvbits(WALL, LEN_INDEX, v, POS_INDEX);
            }
    set_walls(o, lenwwtop, lz - 7);
    set_walls(o, lz - 6, lz - 1);
    for (int z = 6; z <= len - 1; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                if (is_wall(*v) || !dia_kind(x, y, z)) continue;
                *v = (int32_t)((uint32_t)*v | (1u << POS_SI) | (1u << POS_OCC));
            }
    coor_pass(o, 0, lx - 1, 0, ly - 1, 6, lenwwtop + 9, 1);
    list_pass(o, 0, lx - 1, 0, ly - 1, 6, lenwwtop + 9, 1);
}

/* SetTrenchSi, MS/initial/SetTrenchSi.f:22-338 (InitSt ST, MS/main.f:265-266):
 * temperature T(z) = INT(Tbottom + (Ttop - Tbottom) z / (Len3 - 1)) below
 * Len3 and INT(Ttop) above, on every grid point; walls at z = 0..3 and
 * LenZ-4..LenZ-1; Si bulk (coor 4) at z = 4..20; Si at z = 21..Len3-1 except
 * the trench |x - Lenh| <= Len - (Len3 - z) cot(angle), Len2 < z < Len3; then
 * the closing passes over z = 21..Len3+9.  Pi is the reference's
 * REAL(8) :: Pi initialised from a default-REAL literal, i.e. single
 * precision.  With Ttop = Tbottom the tables are interpolated once at Ttop. */
/* With sic it is SetTrench (MS/initial/SetTrench.f:23-283, InitSt 'T'): no
 * temperatures and no walls, the substrate from z = 0, C on the second
 * sublattice and vertical trench sides (|x - Lenh| <= Len). */
static void set_trench(ora_t *o, int len, int len2, int len3, int sic)
{
    int lx = o->lx, ly = o->ly, lz = o->lz;
    const double pi = (double)3.1415926535897932384626433832795028841971f;
    double arad = o->st_angle * pi / 180.0;
    int lenh = lx / 2 - 1;
    int site[3], nextn[4][3];
    lg(o, " %d %d %d\n", lenh, len, len3);
    for (int z = 0; z < lz && !sic; z++) {
        int t = z < len3 ? (int)(o->st_tbottom + (o->st_ttop - o->st_tbottom) * z / (len3 - 1)) : (int)o->st_ttop;
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) mvbits(t, LEN_T, &o->latt[lidx(o, x, y, z)], POS_T);
    }
    if (o->st_fixed && !sic) {
        st_interp(o, (int)o->st_ttop);
        for (int sp = 0; sp < NCRYSTAL_MAX; sp++) {
            double *e = &o->ptransE[sp][0][0][0][0][0][0];
            const double *lo = &o->st_E[o->st_lo][sp][0][0][0][0][0][0], *hi = &o->st_E[o->st_hi][sp][0][0][0][0][0][0];
            for (int k = 0; k < 4096; k++) e[k] = st_mix(o, lo[k], hi[k]);
            for (int c = 0; c < 3; c++) o->ptransD[sp][c] = st_mix(o, o->st_D[o->st_lo][sp][c], o->st_D[o->st_hi][sp][c]);
        }
    }
    if (!sic) {
        set_walls(o, 0, 3);
        set_walls(o, lz - 4, lz - 1);
    }
    for (int z = sic ? 0 : 4; z <= 20; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int k = dia_kind(x, y, z);
                if (!k) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                *v = (int32_t)((uint32_t)*v | (1u << (sic && k == 2 ? POS_C : POS_SI)) | (1u << POS_OCC));
                mvbits(4, LEN_COOR, v, POS_COOR);
                site[0] = x; site[1] = y; site[2] = z;
                std_neighbours(o, site, k == 1 ? 0 : 4, nextn);
                add_bulk(o, site, nextn);
            }
    for (int z = 21; z <= len3 - 1; z++) {
        double half = sic ? (double)len : (double)len - (double)(len3 - z) * cos(arad) / sin(arad);
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int k = dia_kind(x, y, z);
                if (!k) continue;
                if ((double)abs(x - lenh) <= half && z > len2 && z < len3) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                *v = (int32_t)((uint32_t)*v | (1u << (sic && k == 2 ? POS_C : POS_SI)) | (1u << POS_OCC));
            }
    }
    coor_pass(o, 0, lx - 1, 0, ly - 1, 21, len3 + 9, 0);
    list_pass(o, 0, lx - 1, 0, ly - 1, 21, len3 + 9, 0);
}

/* SetCAD, MS/initial/SetCAD.f:24-421 (fresh start), for InitSt 'LA' after
 * SetT (MS/initial/SetT.f:25-50) and for InitSt 'IN' (MS/main.f:279-280).
 * LA: geometry id per layer z (`la_geo[z]`, 1 = Si, 10 = wall/air, as
 * LattGeo; a layer-uniform geometry) and the temperature (K) of the grid
 * points whose coordinates are all multiples of 3,
 * `tsub[((z/3)*(ly/3) + y/3)*(lx/3) + x/3]` (TempStat; 10 marks a wall and
 * is not stored); the Si sites are kept according to the nucleus rule
 * (Homogeneous T/F).  IN: geometry id per site (`cad_geo[(z*ly + y)*lx + x]`),
 * every Si site of id 1 occupied.  Only NCrystal = 1, no alloy (the
 * reference draws the alloy species from the compiler's RAND stream). */
static void set_cad(ora_t *o, int la)
{
    int lx = o->lx, ly = o->ly, lz = o->lz, nx3 = lx / 3, ny3 = ly / 3;
    if (la) {   /* SetT */
        const int16_t *tsub = o->la_tsub;
        for (int z = 0; z < lz; z += 3)
            for (int y = 0; y < ly; y += 3)
                for (int x = 0; x < lx; x += 3) {
                    int t = tsub[((size_t)(z / 3) * ny3 + y / 3) * nx3 + x / 3];
                    if (t != 10) mvbits(t, LEN_T, &o->latt[lidx(o, x, y, z)], POS_T);
                }
    }
    /* walls of SetCAD.f:137-153 and the geometry of :160-236 */
    for (int z = 0; z < lz; z++) {
        int edge = z <= 3 || z >= lz - 4;
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int id = la ? o->la_geo[z] : o->cad_geo[((size_t)z * ly + y) * lx + x];
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                if (edge || id == 10) {
                    *v = (int32_t)((uint32_t)*v | (1u << POS_OCC));
                    mvbits(WALL, LEN_INDEX, v, POS_INDEX);
                } else if (id == 1 && dia_kind(x, y, z)) {
                    int occ = 1;
                    if (!la) {
                    } else if (o->homogeneous[0] == 'T') {
                        occ = z <= lz - (int)((o->len_vac + o->len_nuc) / o->sf);
                    } else {
                        int x0 = lx / 2, y0 = ly / 2, z0 = lz - (int)(o->len_vac / o->sf);
                        long d2 = (long)(x - x0) * (x - x0) + (long)(y - y0) * (y - y0) + (long)(z - z0) * (z - z0);
                        occ = d2 > (long)((o->len_nuc / o->sf) * (o->len_nuc / o->sf));
                    }
                    if (occ) *v = (int32_t)((uint32_t)*v | (1u << POS_OCC) | (1u << POS_SI));
                }
            }
    }
    int site[3], nextn[4][3];
    /* coordinations, removal of isolated atoms (SetCAD.f:241-341) */
    for (int z = 0; z < lz; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                if (ibits(*v, POS_INDEX, LEN_INDEX) == WALL) continue;
                int k = dia_kind(x, y, z);
                if (!k) continue;
                site[0] = x; site[1] = y; site[2] = z;
                std_neighbours(o, site, k == 1 ? 0 : 4, nextn);
                int occ = ibits(*v, POS_OCC, LEN_OCC), coor = 0;
                for (int i = 0; i < 4; i++) {
                    int32_t w = *LC(o, nextn[i]);
                    int occn = ibits(w, POS_OCC, LEN_OCC);
                    if (occ > 0) {
                        if (occn > 0) coor++;
                    } else if (occn > 0 && ibits(w, POS_INDEX, LEN_INDEX) != WALL) {
                        coor++;
                    }
                }
                if (occ != 0 && coor == 0) {
                    int t = ibits(*v, POS_T, LEN_T);
                    *v = 0;
                    mvbits(t, LEN_T, v, POS_T);
                    for (int i = 0; i < 4; i++) {
                        int32_t *w = LC(o, nextn[i]);
                        int cn = ibits(*w, POS_COOR, LEN_COOR) - 1;
                        if (cn < 0) cn = 0;
                        mvbits(cn, LEN_COOR, w, POS_COOR);
                    }
                } else {
                    mvbits(coor, LEN_COOR, v, POS_COOR);
                }
            }
    /* lists and first rates (SetCAD.f:344-421) */
    int nbuff[3] = {0, 0, 0};
    for (int z = 0; z < lz; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int32_t v = o->latt[lidx(o, x, y, z)];
                if (ibits(v, POS_INDEX, LEN_INDEX) == WALL) continue;
                int k = dia_kind(x, y, z);
                if (!k) continue;
                site[0] = x; site[1] = y; site[2] = z;
                std_neighbours(o, site, k == 1 ? 0 : 4, nextn);
                int occ = ibits(v, POS_OCC, LEN_OCC), coor = ibits(v, POS_COOR, LEN_COOR);
                int index_event;
                double prob;
                if (occ == 0) {
                    if (coor == 0) continue;
                    if (coor == 1) {
                        for (int i = 0; i < 4; i++) {
                            int32_t w = *LC(o, nextn[i]);
                            if (ibits(w, POS_OCC, LEN_OCC) != 0 && ibits(w, POS_INDEX, LEN_INDEX) != WALL)
                                cp3(nbuff, nextn[i]);
                            nextn[i][0] = nextn[i][1] = nextn[i][2] = 0;
                        }
                        cp3(nextn[0], nbuff);
                    }
                    if (coor == 4) {
                        add_void(o, site, nextn);
                    } else {
                        get_prob_ini(o, 0, 0, coor, site, nextn, &index_event, &prob);
                        add_mc(o, site, nextn, index_event, prob);
                    }
                } else if (coor <= 3) {
                    get_prob_ini(o, 1, ibits(v, POS_SIC, LEN_SIC), coor, site, nextn, &index_event, &prob);
                    add_mc(o, site, nextn, index_event, prob);
                } else {
                    add_bulk(o, site, nextn);
                }
            }
}

int ora_set_la_input(ora_t *o, const int8_t *geo, const int16_t *tsub)
{
    if (setjmp(o->jb)) return -1;
    if (strcmp(o->init_st, "LA")) ora_fail(o, "LA input given for InitSt %s", o->init_st);
    if (o->ncrystal != 1) ora_fail(o, "the LA initializer is restated for NCrystal = 1");
    if (o->lx % 3 || o->ly % 3 || o->lz % 3) ora_fail(o, "box sides must be multiples of 3");
    size_t nt = (size_t)(o->lx / 3) * (o->ly / 3) * (o->lz / 3);
    free(o->la_geo);
    free(o->la_tsub);
    o->la_geo = (int8_t *)malloc((size_t)o->lz);
    o->la_tsub = (int16_t *)malloc(nt * sizeof(int16_t));
    if (!o->la_geo || !o->la_tsub) ora_fail(o, "allocation failed");
    memcpy(o->la_geo, geo, (size_t)o->lz);
    memcpy(o->la_tsub, tsub, nt * sizeof(int16_t));
    return 0;
}

int ora_set_geometry(ora_t *o, const int8_t *geo)
{
    if (setjmp(o->jb)) return -1;
    if (strcmp(o->init_st, "IN")) ora_fail(o, "a per-site geometry is given for InitSt %s", o->init_st);
    size_t n = (size_t)o->lx * o->ly * o->lz;
    free(o->cad_geo);
    o->cad_geo = (int8_t *)malloc(n);
    if (!o->cad_geo) ora_fail(o, "allocation failed");
    memcpy(o->cad_geo, geo, n);
    return 0;
}

/* ============ start.dat parsing (MS/main.f:80-212, SetProbability.f) ============ */
typedef struct {
    FILE *f;
    char line[4096];
    char *tok;       /* cursor into line for list-directed continuation */
} rd_t;

static int rd_line(rd_t *r)
{
    if (!fgets(r->line, sizeof r->line, r->f)) return 0;
    size_t n = strlen(r->line);
    while (n && (r->line[n - 1] == '\n' || r->line[n - 1] == '\r')) r->line[--n] = 0;
    r->tok = r->line;
    return 1;
}

/* list-directed READ of `n` items: starts a new record, continues to the next
 * record when the current one runs out of values. */
static int rd_items(ora_t *o, rd_t *r, int n, char out[][256])
{
    if (!rd_line(r)) ora_fail(o, "start.dat: unexpected end of file");
    for (int k = 0; k < n; k++) {
        for (;;) {
            while (*r->tok && (isspace((unsigned char)*r->tok) || *r->tok == ',')) r->tok++;
            if (*r->tok) break;
            if (!rd_line(r)) ora_fail(o, "start.dat: unexpected end of file");
        }
        int m = 0;
        while (*r->tok && !isspace((unsigned char)*r->tok) && *r->tok != ',' && m < 255) out[k][m++] = *r->tok++;
        out[k][m] = 0;
    }
    return n;
}

static double to_real(const char *s)
{
    char b[256];
    snprintf(b, sizeof b, "%s", s);
    for (char *p = b; *p; p++)
        if (*p == 'd' || *p == 'D') *p = 'e';
    return strtod(b, NULL);
}

/* One block of rate lines (evaporation, deposition, absorption, desorption)
 * into the given tables; log: print the maxElines line. */
static void read_rate_block(ora_t *o, rd_t *r, double (*pE)[4][4][4][4][4][4], double (*pD)[3], int log)
{   /* SetProbability, MS/mcevent/SetProbability.f:21-143 */
    static const int maxe[4][4] = {   /* [ncov][ncrystal] */
        {0, 3, 18, 57}, {0, 9, 50, 150}, {0, 19, 100, 288}, {0, 34, 172, 480}};
    memset(pE, 0, sizeof(double) * NCRYSTAL_MAX * 4096);
    if (o->ncrystal < 1 || o->ncrystal > 3 || o->ncov < 0 || o->ncov > 3)
        ora_fail(o, "ERROR NOT IMPLEMENTED: NCrystal and NCov must be <= 3 3");
    int maxlines = maxe[o->ncov][o->ncrystal];
    if (log) lg(o, " maxElines %d\n", maxlines);
    char it[3][256];
    for (int i = 0; i < maxlines; i++) {
        rd_items(o, r, 3, it);
        int indsp = atoi(it[0]);
        long elind = atol(it[1]);
        double val = to_real(it[2]);
        if (indsp > o->ncrystal || indsp < 1) ora_fail(o, "ERROR: 1st index in evap prob must be <= NCrystal");
        int ind[6] = {0, 0, 0, 0, 0, 0};
        long p10;
        for (int j = 1; j <= o->ncrystal; j++) {
            p10 = 1;
            for (int q = 0; q < o->ncrystal + o->ncov - j; q++) p10 *= 10;
            ind[j - 1] = (int)((elind / p10) % 10);
        }
        for (int j = o->ncrystal + 1; j <= o->ncrystal + o->ncov; j++) {
            p10 = 1;
            for (int q = 0; q < o->ncrystal + o->ncov - j; q++) p10 *= 10;
            ind[NCRYSTAL_MAX + j - o->ncrystal - 1] = (int)((elind / p10) % 10);
        }
        for (int j = 0; j < 6; j++)
            if (ind[j] > 3) ora_fail(o, "evaporation index digit > 3");
        pE[indsp - 1][ind[0]][ind[1]][ind[2]][ind[3]][ind[4]][ind[5]] = val;
    }
    for (int j = 0; j < o->ncrystal * 3; j++) {
        rd_items(o, r, 3, it);
        int indsp = atoi(it[0]), el = atoi(it[1]);
        if (indsp > o->ncrystal || indsp < 1 || el < 1 || el > 3) ora_fail(o, "ERROR: 1st index in depo prob block must be <= NCrystal");
        pD[indsp - 1][el - 1] = to_real(it[2]);
    }
    for (int j = 0; j < o->ncov * 3; j++) {
        rd_items(o, r, 3, it);
        int indsp = atoi(it[0]), el = atoi(it[1]);
        if (indsp <= o->ncrystal || indsp > o->ncrystal + o->ncov || el < 0 || el > 3) ora_fail(o, "ERROR: absorption index");
        o->ptransAbs[indsp - o->ncrystal - 1][el] = to_real(it[2]);
    }
    for (int j = 0; j < o->ncov * 3; j++) {
        rd_items(o, r, 3, it);
        int indsp = atoi(it[0]), el = atoi(it[1]);
        if (indsp <= o->ncrystal || indsp > o->ncrystal + o->ncov || el < 0 || el > 3) ora_fail(o, "ERROR: desorption index");
        o->ptransDes[indsp - o->ncrystal - 1][el] = to_real(it[2]);
    }
}

static void set_probability(ora_t *o, rd_t *r)
{   /* SetProbability.f:21-143 */
    read_rate_block(o, r, o->ptransE, o->ptransD, 1);
}

/* SetProbabilityFromField, MS/mcevent/SetProbabilityFromField.f:23-171: the
 * table file named on the next line of start.dat: ntemp, nprob, then per
 * temperature its value and one block of rate lines. */
static void set_probability_from_field(ora_t *o, rd_t *r, const char *startdat)
{
    if (!rd_line(r)) ora_fail(o, "start.dat: missing probability table file name");
    char name[4096];
    snprintf(name, sizeof name, "%s", r->line);
    for (char *e = name + strlen(name); e > name && isspace((unsigned char)e[-1]); e--) e[-1] = 0;
    rd_t t;
    memset(&t, 0, sizeof t);
    t.f = fopen(name, "r");
    if (!t.f && name[0] != '/') {              /* relative to the start.dat's directory */
        char alt[8192];
        const char *sl = strrchr(startdat, '/');
        if (sl) {
            snprintf(alt, sizeof alt, "%.*s/%s", (int)(sl - startdat), startdat, name);
            t.f = fopen(alt, "r");
        }
    }
    if (!t.f) ora_fail(o, "cannot open probability table %s", name);
    char it[2][256];
    rd_items(o, &t, 1, it);
    int n = atoi(it[0]);
    rd_items(o, &t, 1, it);                    /* nprob, unused by the reference too */
    if (n < 1 || n > 300) { fclose(t.f); ora_fail(o, "ntemp %d outside 1..300", n); }
    o->st_n = n;
    o->st_E = (double (*)[NCRYSTAL_MAX][4][4][4][4][4][4])calloc((size_t)n, sizeof *o->st_E);
    o->st_D = (double (*)[NCRYSTAL_MAX][3])calloc((size_t)n, sizeof *o->st_D);
    if (!o->st_E || !o->st_D) { fclose(t.f); ora_fail(o, "allocation failed"); }
    for (int i = 0; i < n; i++) {
        rd_items(o, &t, 1, it);
        o->st_T[i] = atoi(it[0]);
        read_rate_block(o, &t, o->st_E[i], o->st_D[i], i == 0);
    }
    fclose(t.f);
}

static void parse_startdat(ora_t *o, const char *path)
{   /* MS/main.f:80-212 */
    rd_t r;
    memset(&r, 0, sizeof r);
    r.f = fopen(path, "r");
    if (!r.f) ora_fail(o, "cannot open %s", path);
    char it[8][256];
    rd_items(o, &r, 2, it);
    o->ncrystal = atoi(it[0]);
    o->ncov = atoi(it[1]);
    if (o->ncrystal > NCRYSTAL_MAX || o->ncrystal < 1) { fclose(r.f); ora_fail(o, "ERR NOT IMPLEMENTED: NCrystal must be <= 3"); }
    rd_items(o, &r, o->ncrystal, it);
    for (int i = 0; i < o->ncrystal; i++) o->list_crystal[i] = atoi(it[i]);
    if (o->ncov > 0 && o->ncov <= NCOV_MAX) {
        rd_items(o, &r, o->ncov, it);
        for (int i = 0; i < o->ncov; i++) o->list_cov[i] = atoi(it[i]);
    } else if (o->ncov != 0) {
        fclose(r.f);
        ora_fail(o, "ERR NOT IMPLEMENTED: NCov must be <= 3");
    }
    rd_items(o, &r, 1, it);
    snprintf(o->init_st, sizeof o->init_st, "%.2s", it[0]);
    if (!strcmp(o->init_st, "FF")) {
        rd_items(o, &r, 4, it);
        o->len1 = atoi(it[0]); o->len2 = atoi(it[1]); o->len3 = atoi(it[2]); o->len4 = atoi(it[3]);
    } else if (!strcmp(o->init_st, "LA")) {    /* MS/main.f:118-138 */
        if (o->ncov > 0) { fclose(r.f); ora_fail(o, "ERR NOT IMPLEMENTED: NCov=0 for LA"); }
        if (!rd_line(&r) || !rd_line(&r)) { fclose(r.f); ora_fail(o, "start.dat: missing LA file names"); }
        rd_items(o, &r, 1, it); o->Tm = to_real(it[0]);
        rd_items(o, &r, 1, it); o->P0 = to_real(it[0]);
        rd_items(o, &r, 1, it); o->sigma = to_real(it[0]);
        rd_items(o, &r, 1, it); o->Tflex = to_real(it[0]);
        rd_items(o, &r, 1, it); o->len_vac = to_real(it[0]);
        rd_items(o, &r, 1, it); o->len_nuc = to_real(it[0]);
        rd_items(o, &r, 1, it); snprintf(o->homogeneous, sizeof o->homogeneous, "%.1s", it[0]);
    } else if (!strcmp(o->init_st, "IN")) {     /* MS/main.f:116-117: the geometry file name */
        if (!rd_line(&r)) { fclose(r.f); ora_fail(o, "start.dat: missing geometry file name"); }
    } else if (!strcmp(o->init_st, "ST")) {     /* MS/main.f:109-115 */
        rd_items(o, &r, 6, it);
        o->len1 = atoi(it[0]); o->len2 = atoi(it[1]); o->len3 = atoi(it[2]);
        o->st_angle = to_real(it[3]); o->st_ttop = to_real(it[4]); o->st_tbottom = to_real(it[5]);
        lg(o, " Temperature on top in Kelvin: %.17g\n", o->st_ttop);
        lg(o, " Temperature on bottom in Kelvin: %.17g\n", o->st_tbottom);
        o->st = 1;
        o->st_fixed = o->st_ttop == o->st_tbottom;
        if (o->ncov != 0) { fclose(r.f); ora_fail(o, "InitSt ST with coverage species is not restated"); }
    } else if (!strcmp(o->init_st, "SH")) {     /* MS/main.f:116-117: READ(IPF,'(A)') the file name */
        if (!rd_line(&r)) { fclose(r.f); ora_fail(o, "start.dat: missing shape file name"); }
        const char *b = r.line;
        while (*b && isspace((unsigned char)*b)) b++;
        size_t m = strlen(b);
        while (m && isspace((unsigned char)b[m - 1])) m--;
        if (m >= sizeof o->shapefile) { fclose(r.f); ora_fail(o, "shape file name too long"); }
        memcpy(o->shapefile, b, m);
        o->shapefile[m] = 0;
    } else {
        rd_items(o, &r, 3, it);
        o->len1 = atoi(it[0]); o->len2 = atoi(it[1]); o->len3 = atoi(it[2]);
    }
    int sige = (o->ncrystal >= 2 && o->list_crystal[0] == 14 && o->list_crystal[1] == 32 &&
                (o->ncrystal == 2 || o->list_crystal[2] == 5));
    if (sige) {
        rd_items(o, &r, 1, it);
        o->alloyfraction = to_real(it[0]);
    }
    rd_items(o, &r, 1, it);
    o->ptrans_zig = to_real(it[0]);
    rd_items(o, &r, 1, it);
    o->sf = to_real(it[0]);
    rd_items(o, &r, 1, it);
    snprintf(o->exit_strategy, sizeof o->exit_strategy, "%.4s", it[0]);
    if (!strcmp(o->exit_strategy, "Iter")) {
        rd_items(o, &r, 1, it); o->max_iter = atoll(it[0]);
        rd_items(o, &r, 1, it); o->out_molmol = atoll(it[0]);
    } else if (!strcmp(o->exit_strategy, "Time")) {
        rd_items(o, &r, 1, it); o->max_time = to_real(it[0]);
        rd_items(o, &r, 1, it); o->out_time = to_real(it[0]);
    }
    rd_items(o, &r, 1, it);
    snprintf(o->run_type, sizeof o->run_type, "%.2s", it[0]);
    rd_items(o, &r, 1, it);
    o->idum = atoi(it[0]);
    rd_items(o, &r, 1, it);
    snprintf(o->save_final, sizeof o->save_final, "%.2s", it[0]);
    if (!strcmp(o->save_final, "T")) {
        if (!rd_line(&r)) ora_fail(o, "start.dat: missing restart file name");
        snprintf(o->restartfile, sizeof o->restartfile, "%s", r.line);
    }
    rd_items(o, &r, 1, it);
    snprintf(o->save_coo, sizeof o->save_coo, "%.2s", it[0]);
    if (!strcmp(o->save_coo, "T")) {
        if (!rd_line(&r)) ora_fail(o, "start.dat: missing coo file name");
        snprintf(o->coofile, sizeof o->coofile, "%s", r.line);
    }
    if (o->st) set_probability_from_field(o, &r, path);   /* MS/main.f:215-219 */
    else set_probability(o, &r);
    fclose(r.f);
}

/* ============ output: MS/inpout/ ============ */
/* Fortran Ew.d (0.ddddE+xx) */
static void fmt_e(char *out, double v, int w, int d)
{
    char m[64], b[64];
    if (v == 0.0) {
        snprintf(b, sizeof b, "0.%0*dE+00", d, 0);
    } else {
        snprintf(m, sizeof m, "%.*e", d - 1, fabs(v));
        /* m = "D.DDDDe+XX" */
        char digits[64];
        int nd = 0;
        char *p = m;
        digits[nd++] = *p++;
        if (*p == '.') p++;
        while (*p && *p != 'e') digits[nd++] = *p++;
        digits[nd] = 0;
        int ex = atoi(p + 1) + 1;
        snprintf(b, sizeof b, "%s0.%sE%c%02d", v < 0 ? "-" : "", digits, ex < 0 ? '-' : '+', abs(ex));
    }
    snprintf(out, 64, "%*s", w, b);
}

static void fmt_header(char *out, size_t n, int count, double time, int64_t iter)
{   /* FORMAT (1x,i8,1x,a,1x,a,1x,e15.8,1x,a,1x,i12), WriteMolMolXYZFile.f:166 */
    char e[64];
    fmt_e(e, time, 15, 8);
    snprintf(out, n, " %8d angstroem KMC-time: %s Iter: %12lld\n", count, e, (long long)iter);
}

static void fmt_periodic(char *out, size_t n, ora_t *o)
{   /* FORMAT (1x,a,3(1x,e15.8)), WriteMolMolXYZFile.f:169 */
    char a[64], b[64], c[64];
    fmt_e(a, o->sf * (double)o->lx, 15, 8);
    fmt_e(b, o->sf * (double)o->ly, 15, 8);
    fmt_e(c, o->sf * (double)o->lz, 15, 8);
    snprintf(out, n, " periodic %s %s %s\n", a, b, c);
}

static void wr_atom(FILE *f, const char *sym, ora_t *o, int x, int y, int z)
{   /* FORMAT('Si ',F10.5,' ',F10.5,' ',F10.5,'  ',F6.2) with 3 items */
    fprintf(f, "%s %10.5f %10.5f %10.5f  \n", sym, o->sf * (double)x, o->sf * (double)y, o->sf * (double)z);
}

static const char *species_sym(ora_t *o, int iat)
{
    if (iat == 1) return "Si";
    int z = o->list_crystal[iat - 1];
    if (z == 6) return "C";
    if (z == 32) return "Ge";
    if (z == 5) return "B";
    return NULL;
}

/* WriteMolMolXYZFile, MS/inpout/WriteMolMolXYZFile.f:22-406.  f_xyz is the
 * main frame, f_d the non-epitaxial bulk list, f_v the vacancies, f_w the
 * SiC wrong-bond list (may be NULL). */
static void write_xyz_files(ora_t *o, FILE *f_xyz, FILE *f_d, FILE *f_v, FILE *f_w, double time, int64_t iter)
{
    char hdr[256], per[256];
    int num_at = 0, num_cov = 0, noepi_bulk = 0;
    for (int z = 1; z <= o->lz - 1; z++)
        for (int y = 0; y < o->ly; y++)
            for (int x = 0; x < o->lx; x++) {
                int32_t v = o->latt[lidx(o, x, y, z)];
                int covind = ibits(v, POS_INDEX, LEN_INDEX);
                if (covind != WALL) {
                    int occ = ibits(v, POS_OCC, LEN_OCC), coo = ibits(v, POS_COOR, LEN_COOR);
                    if (occ == 1 && coo <= 3) num_at++;
                    else if (occ == 0 && covind != 0) num_cov++;
                }
            }
    for (int z = 0; z <= o->lz - 1; z++)
        for (int y = 0; y < o->ly; y++)
            for (int x = 0; x < o->lx; x++) {
                int32_t v = o->latt[lidx(o, x, y, z)];
                if (ibits(v, POS_OCC, LEN_OCC) == 1 && ibits(v, POS_COOR, LEN_COOR) == 4 && !dia_kind(x, y, z))
                    noepi_bulk++;
            }
    lg(o, " %d\n", noepi_bulk);
    fmt_periodic(per, sizeof per, o);
    if (f_d) {
        fmt_header(hdr, sizeof hdr, noepi_bulk, time, iter);
        fputs(hdr, f_d);
        fputs(per, f_d);
        for (int z = 0; z <= o->lz - 1; z++)
            for (int y = 0; y < o->ly; y++)
                for (int x = 0; x < o->lx; x++) {
                    int32_t v = o->latt[lidx(o, x, y, z)];
                    if (ibits(v, POS_OCC, LEN_OCC) == 1 && ibits(v, POS_COOR, LEN_COOR) == 4 && !dia_kind(x, y, z)) {
                        int iat = ibits(v, POS_SIC, LEN_SIC);
                        if (iat == 1) wr_atom(f_d, "Ge", o, x, y, z);
                        if (iat == 2) wr_atom(f_d, "B", o, x, y, z);
                        if (iat == 3) wr_atom(f_d, "Cl", o, x, y, z);
                    }
                }
    }
    if (f_xyz) {
        fmt_header(hdr, sizeof hdr, num_at + o->num_void + num_cov, time, iter);
        fputs(hdr, f_xyz);
        fputs(per, f_xyz);
        for (int z = 0; z <= o->lz - 1; z++)
            for (int y = 0; y < o->ly; y++)
                for (int x = 0; x < o->lx; x++) {
                    int32_t v = o->latt[lidx(o, x, y, z)];
                    int iat = ibits(v, POS_SIC, LEN_SIC);
                    int coo = ibits(v, POS_COOR, LEN_COOR);
                    int covind = ibits(v, POS_INDEX, LEN_INDEX);
                    if (covind == 1) wr_atom(f_xyz, "H", o, x, y, z);
                    if (covind == 17) wr_atom(f_xyz, "Cl", o, x, y, z);
                    if (iat >= 1 && iat <= 3 && coo <= 3) {
                        if (iat > o->ncrystal) ora_fail(o, "ERR: IAt=%d should not happen", iat);
                        const char *sym = species_sym(o, iat);
                        if (!sym) ora_fail(o, "ERROR: 2nd crystal specie can only be C/Ge/B");
                        wr_atom(f_xyz, sym, o, x, y, z);
                    }
                }
        for (int i = 1; i <= o->num_void; i++)
            wr_atom(f_xyz, "O", o, o->voids[i].xyz[0], o->voids[i].xyz[1], o->voids[i].xyz[2]);
    }
    if (f_v) {
        fprintf(f_v, " %8d angstroem\n", o->num_void);
        fputs(per, f_v);
        for (int i = 1; i <= o->num_void; i++) {
            int x = o->voids[i].xyz[0], y = o->voids[i].xyz[1], z = o->voids[i].xyz[2];
            if (o->ncov == 0 && o->ncrystal == 2 && o->list_crystal[1] == 6) {
                int iat = 0;
                for (int j = 0; j < 4; j++) iat += ibits(*LC(o, o->voids[i].nn[j]), POS_SIC, LEN_SIC);
                const char *lbl = NULL;
                if (iat == 4) lbl = "Mg %10.5f %10.5f %10.5f # CV (C vacancy)\n";
                else if (iat == 8) lbl = "He %10.5f %10.5f %10.5f # SV (Si vacancy)\n";
                else if (iat == 7) lbl = "Ne %10.5f %10.5f %10.5f # SAV (Si antisite vac)\n";
                else if (iat == 5) lbl = "Be %10.5f %10.5f %10.5f # CAV (C antisite vac)\n";
                else if (iat == 6) lbl = "Ar %10.5f %10.5f %10.5f # XV (near 2C and 2Si)\n";
                else ora_fail(o, "ERROR: Weird Defect type was formed...ABORTING");
                fprintf(f_v, lbl, o->sf * x, o->sf * y, o->sf * z);
            } else {
                wr_atom(f_v, "O", o, x, y, z);
            }
        }
    }
    /* SiC "wrong" sites, :264-398 (mutates and then restores LattCoo with
     * the type of the LAST buffered site, as the reference does). */
    int sic = 0;
    if (o->ncrystal == 2)
        for (int k = 0; k < NCRYSTAL_MAX; k++)
            if (o->list_crystal[k] == 6) sic = 1;
    if (sic) {
        int num_is_wrong = 0;
        for (int z = 1; z <= o->lz - 1; z++)
            for (int y = 0; y < o->ly; y++)
                for (int x = 0; x < o->lx; x++) {
                    int32_t *v = &o->latt[lidx(o, x, y, z)];
                    if (ibits(*v, POS_INDEX, LEN_INDEX) == WALL) continue;
                    if (ibits(*v, POS_OCC, LEN_OCC) == 1 && ibits(*v, POS_COOR, LEN_COOR) == 4) {
                        int ind = o->lind[lidx(o, x, y, z)];
                        int iat = ibits(*v, POS_SIC, LEN_SIC);
                        int nc = 0;
                        for (int i = 0; i < 4; i++) {
                            int32_t w = *LC(o, o->bulk[ind].nn[i]);
                            if (iat == 1) nc += ibits(w, POS_C, 1);
                            else if (iat == 2) nc += ibits(w, POS_SI, 1);
                        }
                        if (nc == 0) {
                            num_is_wrong++;
                            if (num_is_wrong >= o->atbuf_cap) {
                                int nc2 = o->atbuf_cap * 2 + 64;
                                o->atbuf = (atbuf_t *)realloc(o->atbuf, (size_t)nc2 * sizeof(atbuf_t));
                                o->atbuf_cap = nc2;
                            }
                            atbuf_t *b = &o->atbuf[num_is_wrong];
                            b->xyz[0] = x; b->xyz[1] = y; b->xyz[2] = z;
                            if (iat == 1) {
                                *v = (int32_t)(((uint32_t)*v & ~(1u << POS_SI)) | (1u << POS_C));
                                b->ind_atype = 1;
                            } else {
                                *v = (int32_t)(((uint32_t)*v & ~(1u << POS_C)) | (1u << POS_SI));
                                b->ind_atype = 2;
                            }
                        }
                    }
                }
        int num_at_wrong = 0;
        for (int pass = 0; pass < 2; pass++) {
            if (pass == 1 && f_w) {
                fprintf(f_w, " %8d angstroem\n", num_at_wrong);
                fputs(per, f_w);
            }
            for (int z = 1; z <= o->lz - 1; z++)
                for (int y = 0; y < o->ly; y++)
                    for (int x = 0; x < o->lx; x++) {
                        int32_t v = o->latt[lidx(o, x, y, z)];
                        if (ibits(v, POS_OCC, LEN_OCC) == 1 && ibits(v, POS_COOR, LEN_COOR) == 4) {
                            int ind = o->lind[lidx(o, x, y, z)];
                            int iat = ibits(v, POS_SIC, LEN_SIC);
                            int nc = 0;
                            for (int i = 0; i < 4; i++) {
                                int32_t w = *LC(o, o->bulk[ind].nn[i]);
                                if (iat == 1) nc += ibits(w, POS_C, 1);
                                else if (iat == 2) nc += ibits(w, POS_SI, 1);
                            }
                            if (nc == 3) {
                                if (pass == 0) num_at_wrong++;
                                else if (f_w) {
                                    if (iat == 1) wr_atom(f_w, "Si", o, x, y, z);
                                    if (iat == 2) wr_atom(f_w, "C", o, x, y, z);
                                }
                            }
                        }
                    }
            if (pass == 0) lg(o, " NumAtWrong: %d\n", num_at_wrong);
        }
        for (int i = 1; i <= num_is_wrong; i++) {
            atbuf_t *b = &o->atbuf[i];
            int32_t *v = &o->latt[lidx(o, b->xyz[0], b->xyz[1], b->xyz[2])];
            if (o->atbuf[num_is_wrong].ind_atype == 1)
                *v = (int32_t)(((uint32_t)*v & ~(1u << POS_C)) | (1u << POS_SI));
            else
                *v = (int32_t)(((uint32_t)*v & ~(1u << POS_SI)) | (1u << POS_C));
        }
    }
}

/* GetOutputFileName, MS/inpout/GetOutputFileName.f:22-81: 'I' followed by
 * the first 8 of the 9 digits of Iout*10 (CHARACTER(Len=9) truncation). */
static void output_name(ora_t *o, int64_t iout, char base[16])
{
    int64_t t = iout * 10;
    if (t >= 1000000000LL) ora_fail(o, "GetOutputFileName:: Iter can not be represented");
    char d[32];
    snprintf(d, sizeof d, "%09lld", (long long)t);
    base[0] = 'I';
    memcpy(base + 1, d, 8);
    base[9] = 0;
}

/* WriteMolMolSource, MS/inpout/WriteMolMolSource.f:22-112 */
static void write_molmol_source(ora_t *o, const char *outdir, double time, int64_t iter, int64_t iout)
{
    char base[16], path[4096];
    output_name(o, iout, base);
    lg(o, " %s\n", base);
    if (!outdir) return;
    FILE *fx, *fd, *fv, *fw = NULL, *fs;
    snprintf(path, sizeof path, "%s/%s.xyz", outdir, base);
    fx = fopen(path, "w");
    snprintf(path, sizeof path, "%s/%s_d.xyz", outdir, base);
    fd = fopen(path, "w");
    snprintf(path, sizeof path, "%s/%s_v.xyz", outdir, base);
    fv = fopen(path, "w");
    int sic = 0;
    if (o->ncrystal == 2)
        for (int k = 0; k < NCRYSTAL_MAX; k++)
            if (o->list_crystal[k] == 6) sic = 1;
    if (sic) {
        snprintf(path, sizeof path, "%s/%s_w.xyz", outdir, base);
        fw = fopen(path, "w");
    }
    if (!fx || !fd || !fv) ora_fail(o, "cannot open output files in %s", outdir);
    write_xyz_files(o, fx, fd, fv, fw, time, iter);
    fclose(fx);
    fclose(fd);
    fclose(fv);
    if (fw) fclose(fw);
    snprintf(path, sizeof path, "%s/%s.src", outdir, base);
    fs = fopen(path, "w");
    if (fs) {
        fprintf(fs, " load xyz %s.xyz\n color temperature\n set background white\n set boundbox true\n"
                    " zoom 140\n rotate x 41\n rotate y 4\n spacefill 2\n color axes black\n wireframe 2\n"
                    " color atom green\n wireframe 12\n color atom purple\n set bondmode and\n", base);
        fclose(fs);
    }
    snprintf(path, sizeof path, "%s/movie.mos", outdir);
    fs = fopen(path, "a");
    if (fs) {
        fprintf(fs, " source    %s.src\n write gif %s.gif\n zap\n", base, base);
        fclose(fs);
    }
}

/* ============ public API ============ */
ora_t *ora_create(const char *startdat_path, const char *numbers_path, int lenx, int leny, int lenz, int num_mc_max)
{
    ora_t *o = (ora_t *)calloc(1, sizeof(ora_t));
    if (!o) return NULL;
    o->lx = lenx; o->ly = leny; o->lz = lenz;
    o->mc_max = num_mc_max > 0 ? num_mc_max : 500000;
    o->bulk_max = 100000000;
    o->void_max = 100000;
    o->iter = 1;
    o->log = NULL;
    if (setjmp(o->jb)) {
        ora_destroy(o);
        return NULL;
    }
    if (lenx <= 0 || leny <= 0 || lenz <= 0) ora_fail(o, "bad box");
    int64_t plane = (int64_t)lenx * leny;
    int64_t n = plane * ((int64_t)lenz + 1 + 2 * ZGUARD);
    o->latt_base = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    o->lind_base = (int32_t *)calloc((size_t)n, sizeof(int32_t));
    if (!o->latt_base || !o->lind_base) ora_fail(o, "lattice allocation failed");
    o->latt = o->latt_base + plane * ZGUARD;
    o->lind = o->lind_base + plane * ZGUARD;
    o->mc = (mcp_t *)calloc((size_t)o->mc_max + 2, sizeof(mcp_t));
    o->bulk_cap = 1 << 16;
    o->bulk = (blk_t *)calloc((size_t)o->bulk_cap, sizeof(blk_t));
    o->voids = (blk_t *)calloc((size_t)o->void_max + 2, sizeof(blk_t));
    o->atbuf_cap = 1024;
    o->atbuf = (atbuf_t *)calloc((size_t)o->atbuf_cap, sizeof(atbuf_t));
    if (!o->mc || !o->bulk || !o->voids || !o->atbuf) ora_fail(o, "list allocation failed");
    if (numbers_path) {
        FILE *f = fopen(numbers_path, "r");
        if (!f) ora_fail(o, "cannot open %s", numbers_path);
        for (int i = 0; i < 1000; i++) {
            float v;
            if (fscanf(f, "%f", &v) != 1) { fclose(f); ora_fail(o, "bad numbers file"); }
            o->numbers[i] = (double)v;
        }
        fclose(f);
        o->have_numbers = 1;
    }
    parse_startdat(o, startdat_path);
    if (o->run_type[0] == 'T' && !o->have_numbers) ora_fail(o, "RunType T needs the test-mode number list");
    allocate_arrays(o);
    return o;
}

void ora_destroy(ora_t *o)
{
    if (!o) return;
    free(o->la_k);
    free(o->la_dk);
    free(o->la_ps);
    free(o->la_kind);
    free(o->la_geo);
    free(o->la_tsub);
    free(o->cad_geo);
    free(o->st_E);
    free(o->st_D);
    free(o->latt_base);
    free(o->lind_base);
    free(o->mc);
    free(o->bulk);
    free(o->voids);
    free(o->atbuf);
    free(o->tree);
    free(o->trace);
    free(o);
}

/* SetShape, MS/initial/SetShape.f:25-436 (InitSt 'SH', called from
 * MS/main.f:281-286).  The point-list file named in start.dat holds NFilled,
 * one skipped record, then NFilled records `sym x y z` (:52-79): every point
 * is occupied; one with z <= 3 or z >= LenZ-4 is a wall, any other is Si for
 * 'Si' and species 2 for 'C' or 'Ge' (sym is CHARACTER(Len=2)).  Then, over
 * z = 4..LenZ-5 in z, y, x order (:98-186), every occupied point takes as
 * neighbours the occupied points of its |d|^2 = 27 shell, scanned dz, dy, dx
 * from -6 to 6 (:87-99, :113-131); with coordination <= 3 it is an MC
 * particle whose neighbours 3 and 4 come from FIND_NN of the first two
 * (:136-143), with 4 a bulk atom.  The reciprocity checks of the MC particles
 * (:277-320) and of the bulk atoms above z = 12 (:325-373) follow, then the
 * ad-voids: each empty neighbour of the MC particles present before that
 * pass gains one coordination per MC neighbour, in list order (:378-431).
 * Two inputs leave the reference undefined and are rejected here: an atom
 * with fewer than two neighbours (FIND_NN of a zero NextND(2)) or more than
 * four (NextND overflows), and a reciprocity check that meets a wall (the
 * wall's LattInd is 0, so ListAdAtom(0) is read). */
static void set_shape(ora_t *o)
{
    int lx = o->lx, ly = o->ly, lz = o->lz;
    rd_t r;
    r.f = fopen(o->shapefile, "r");
    if (!r.f) ora_fail(o, "cannot open the shape file %s", o->shapefile);
    char it[4][256];
    lg(o, " Reading input geometry file (SHAPE): %s\n", o->shapefile);
    rd_items(o, &r, 1, it);
    int nfilled = atoi(it[0]);
    if (!rd_line(&r)) { fclose(r.f); ora_fail(o, "shape file: missing second record"); }
    for (int ia = 0; ia < nfilled; ia++) {
        rd_items(o, &r, 4, it);
        int x = atoi(it[1]), y = atoi(it[2]), z = atoi(it[3]);
        if (x < 0 || x >= lx || y < 0 || y >= ly || z < 0 || z > lz) {
            fclose(r.f);
            ora_fail(o, "shape file: point %d %d %d outside the box", x, y, z);
        }
        int32_t *v = &o->latt[lidx(o, x, y, z)];
        *v = (int32_t)((uint32_t)*v | (1u << POS_OCC));
        char sym[3] = {it[0][0], it[0][0] ? it[0][1] : 0, 0};
        if (z >= lz - 4 || z <= 3) {
            mvbits(WALL, LEN_INDEX, v, POS_INDEX);
        } else if (!strcmp(sym, "Si")) {
            *v = (int32_t)((uint32_t)*v | (1u << POS_SI));
        } else if (!strcmp(sym, "C") || !strcmp(sym, "Ge")) {
            *v = (int32_t)((uint32_t)*v | (1u << POS_C));
        }
    }
    fclose(r.f);
    lg(o, " Done reading input geometry file\n");
    int list[32][3], nlist = 0;
    for (int k = -6; k <= 6; k++)
        for (int j = -6; j <= 6; j++)
            for (int i = -6; i <= 6; i++)
                if (i * i + j * j + k * k == 27) {
                    list[nlist][0] = i; list[nlist][1] = j; list[nlist][2] = k;
                    nlist++;
                }
    int site[3], nextnd[4][3], ns[2][3], buf[3], index_event;
    double prob;
    for (int z = 4; z <= lz - 5; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                if (ibits(*v, POS_OCC, LEN_OCC) == 0) continue;
                site[0] = x; site[1] = y; site[2] = z;
                memset(nextnd, 0, sizeof nextnd);
                int coord = 0;
                for (int i = 0; i < nlist; i++) {
                    int nsite[3] = {x + list[i][0], y + list[i][1], z + list[i][2]};
                    if (nsite[0] >= lx) nsite[0] -= lx;
                    if (nsite[0] < 0) nsite[0] += lx;
                    if (nsite[1] >= ly) nsite[1] -= ly;
                    if (nsite[1] < 0) nsite[1] += ly;
                    if (ibits(*LC(o, nsite), POS_OCC, LEN_OCC) > 0) {
                        if (coord == 4) ora_fail(o, "SetShape: more than four neighbours at %d %d %d", x, y, z);
                        cp3(nextnd[coord], nsite);
                        coord++;
                    }
                }
                mvbits(coord, LEN_COOR, v, POS_COOR);
                if (coord <= 3) {
                    if (coord < 2) ora_fail(o, "SetShape: %d neighbours at %d %d %d", coord, x, y, z);
                    cp3(buf, nextnd[2]);
                    find_nn(nextnd[0], nextnd[1], site, ns, lx, ly);
                    cp3(nextnd[2], ns[0]);
                    cp3(nextnd[3], ns[1]);
                    if (coord == 3) {
                        int check = 1;
                        for (int i = 0; i < 4; i++)
                            if (nextnd[i][0] == buf[0] && nextnd[i][1] == buf[1] && nextnd[i][2] == buf[2]) check = 0;
                        if (check) lg(o, " Coord.eq.3 wrong check Buf %d %d %d\n", buf[0], buf[1], buf[2]);
                    }
                    get_prob_ini(o, 1, ibits(*v, POS_SIC, LEN_SIC), coord, site, nextnd, &index_event, &prob);
                    add_mc(o, site, nextnd, index_event, prob);
                } else {
                    add_bulk(o, site, nextnd);
                }
            }
    /* reciprocal bonds only: MC particles, then bulk atoms above z = 12 */
    for (int pass = 0; pass < 2; pass++) {
        int64_t n0 = pass == 0 ? o->num_mc : o->num_bulk;
        for (int64_t i = 1; i <= n0; i++) {
            int nextn[4][3];
            if (pass == 0) {
                cp3(site, o->mc[i].xyz);
                memcpy(nextn, o->mc[i].nn, sizeof nextn);
            } else {
                cp3(site, o->bulk[i].xyz);
                if (site[2] < 13) continue;
                memcpy(nextn, o->bulk[i].nn, sizeof nextn);
            }
            int32_t *v = LC(o, site);
            int coor = ibits(*v, POS_COOR, LEN_COOR), coorold = coor;
            for (int j = 0; j < 4; j++) {
                int32_t w = *LC(o, nextn[j]);
                if (ibits(w, POS_OCC, LEN_OCC) == 0) continue;
                if (is_wall(w))
                    ora_fail(o, "SetShape: the reciprocity check of %d %d %d meets a wall", site[0], site[1], site[2]);
                int ind = *LI(o, nextn[j]);
                int (*nnn)[3] = ibits(w, POS_COOR, LEN_COOR) == 4 ? o->bulk[ind].nn : o->mc[ind].nn;
                int recipr = 0;
                for (int k = 0; k < 4; k++)
                    if (nnn[k][0] == site[0] && nnn[k][1] == site[1] && nnn[k][2] == site[2]) recipr = 1;
                if (!recipr) coor--;
            }
            if (coor == coorold) continue;
            int ind = *LI(o, site), iat = ibits(*v, POS_SIC, LEN_SIC);
            mvbits(coor, LEN_COOR, v, POS_COOR);
            get_prob(o, 1, iat, 0, coor, site, nextn, &index_event, &prob);
            if (pass == 0) {
                o->mc[ind].ind_event = index_event;
                o->mc[ind].prob = prob;
                update_tree(o, ind, prob);
            } else {
                erase_bulk(o, site);
                add_mc(o, site, nextn, index_event, prob);
            }
        }
    }
    /* the ad-voids */
    int nmc0 = o->num_mc;
    for (int i = 1; i <= nmc0; i++) {
        int nnsite[3];
        cp3(nnsite, o->mc[i].xyz);
        for (int j = 0; j < 4; j++) {
            cp3(site, o->mc[i].nn[j]);
            int32_t *v = LC(o, site);
            if (ibits(*v, POS_OCC, LEN_OCC) != 0) continue;
            int nextn[4][3];
            memset(nextn, 0, sizeof nextn);
            int coor = ibits(*v, POS_COOR, LEN_COOR) + 1;
            if (coor == 1) {
                cp3(nextn[0], nnsite);
                mvbits(coor, LEN_COOR, v, POS_COOR);
                get_prob_ini(o, 0, 0, coor, site, nextn, &index_event, &prob);
                add_mc(o, site, nextn, index_event, prob);
            } else if (coor == 2 || coor == 3) {
                int ind = *LI(o, site);
                memcpy(nextn, o->mc[ind].nn, sizeof nextn);
                if (coor == 2) {
                    cp3(nextn[1], nnsite);
                    find_nn(nextn[0], nextn[1], site, ns, lx, ly);
                    cp3(nextn[2], ns[0]);
                    cp3(nextn[3], ns[1]);
                }
                mvbits(coor, LEN_COOR, v, POS_COOR);
                get_prob_ini(o, 0, 0, coor, site, nextn, &index_event, &prob);
                memcpy(o->mc[ind].nn, nextn, sizeof nextn);
                o->mc[ind].ind_event = index_event;
                o->mc[ind].prob = prob;
                update_tree(o, ind, prob);
            } else {
                ora_fail(o, "Vacancy in the SF setting");
            }
        }
    }
}

/* SetSiCSF, MS/initial/SetSiCSF.f:7-473 (InitSt 'E', MS/main.f:267-272:
 * called with Len1 and the vertex VSF = (Len2, Len3, Len1 - Len2)): a 3C-SiC
 * (001) slab up to z = Len - 1 holding a triangular triple stacking fault.
 * In the region x >= VSF(1), y >= VSF(2), z >= VSF(3) the atoms of two
 * {111} planes per sublattice (Si: (x-Vx)+(y-Vy)-(z-Vz) = 12 and 24, C: 3
 * and 15) are shifted by (+2, +2, +4) and (-2, -2, -4), off the diamond
 * sites.  Then two passes over z = 13..Len+6 in scan order: the first
 * empties atoms with fewer than two neighbours (diamond bonds, or the
 * 32-site |d|^2 = 27 shell when they have fewer than two diamond bonds);
 * the second sets coordinations and builds the lists, an off-grid atom's
 * NextN being its shell neighbours completed by FIND_NN, rates by
 * Get_Prob_Ini.  Then the coordinations are cut to reciprocal bonds, MC
 * atoms first, then bulk atoms of z >= 13 (re-rated by Get_Prob; a bulk atom
 * that changes becomes MC: EraseBulk, AddMC -- over the bulk count at the
 * loop's start, as the Fortran DO evaluates it once), and last the ad-voids
 * of every MC atom's NextN (:432-471). */
static void set_sicsf(ora_t *o, int len, const int vsf[3])
{
    const int lx = o->lx, ly = o->ly;
    const int box_sf = len - vsf[2];
    int shell[32][3], ns = 0;                       /* ListNN, :24-35: k outer, i inner */
    for (int k = -6; k <= 6; k++)
        for (int j = -6; j <= 6; j++)
            for (int i = -6; i <= 6; i++)
                if (i * i + j * j + k * k == 27) {
                    shell[ns][0] = i;
                    shell[ns][1] = j;
                    shell[ns][2] = k;
                    ns++;
                }
    if (vsf[0] + box_sf > lx || vsf[1] + box_sf > ly || box_sf <= 0)
        ora_fail(o, "error SF dimension is not correctly set");
    if (dia_kind(vsf[0], vsf[1], vsf[2]) != 1)
        ora_fail(o, "SF Vertex position in wrong Site %d %d %d %d", vsf[0], vsf[1], vsf[2], len);
    if (len + 9 > o->lz) ora_fail(o, "SetSiCSF reads up to z = Len + 9: LenZ too small");
    int site[3], nextn[4][3];
    /* :56-107: bulk 3C for z = 0..12 */
    for (int z = 0; z <= 12; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int k = dia_kind(x, y, z);
                if (!k) continue;
                int32_t *v = &o->latt[lidx(o, x, y, z)];
                *v = (int32_t)((uint32_t)*v | (1u << (k == 1 ? POS_SI : POS_C)) | (1u << POS_OCC));
                mvbits(4, LEN_COOR, v, POS_COOR);
                site[0] = x; site[1] = y; site[2] = z;
                std_neighbours(o, site, k == 1 ? 0 : 4, nextn);
                add_bulk(o, site, nextn);
            }
    /* :109-163: z = 13..Len-1 with the shifted planes (bits only: IBSET) */
    for (int z = 13; z <= len - 1; z++)
        for (int y = 0; y < ly; y++)
            for (int x = 0; x < lx; x++) {
                int k = dia_kind(x, y, z);
                if (!k) continue;
                const int inside = x >= vsf[0] && y >= vsf[1] && z >= vsf[2];
                const int d = (x - vsf[0]) + (y - vsf[1]) - (z - vsf[2]);
                const int p1 = inside ? d - (k == 1 ? 12 : 3) : -1;
                const int p2 = inside ? d - (k == 1 ? 24 : 15) : -1;
                int tx = x, ty = y, tz = z;
                if (p1 == 0) {
                    if (!(x + 2 < lx && y + 2 < ly && z + 4 < len)) continue;
                    tx = x + 2; ty = y + 2; tz = z + 4;
                } else if (p2 == 0) {
                    if (!(x - 2 > 0 && y - 2 > 0 && z - 4 > 0)) continue;
                    tx = x - 2; ty = y - 2; tz = z - 4;
                }
                int32_t *v = &o->latt[lidx(o, tx, ty, tz)];
                *v = (int32_t)((uint32_t)*v | (1u << (k == 1 ? POS_SI : POS_C)) | (1u << POS_OCC));
            }
    /* the diamond bonds and the shell neighbours of an occupied site (:172-208) */
    int nd[32][3];
    for (int pass = 0; pass < 2; pass++)
        for (int z = 13; z <= len + 6; z++)
            for (int y = 0; y < ly; y++)
                for (int x = 0; x < lx; x++) {
                    int32_t *v = &o->latt[lidx(o, x, y, z)];
                    if (!ibits(*v, POS_OCC, LEN_OCC)) continue;
                    site[0] = x; site[1] = y; site[2] = z;
                    const int sic = ((x / 3 + y / 3 + z / 3) % 4 == 3) ? 4 : 0;
                    std_neighbours(o, site, sic, nextn);
                    int coor = 0, coord = 0, j = 0;
                    for (int i = 0; i < 4; i++)
                        if (ibits(*LC(o, nextn[i]), POS_OCC, LEN_OCC)) coor++;
                    if (coor < 2) {
                        for (int i = 0; i < ns; i++) {
                            int q[3] = {x + shell[i][0], y + shell[i][1], z + shell[i][2]};
                            if (q[0] >= lx) q[0] -= lx;
                            if (q[0] < 0) q[0] += lx;
                            if (q[1] >= ly) q[1] -= ly;
                            if (q[1] < 0) q[1] += ly;
                            if (ibits(*LC(o, q), POS_OCC, LEN_OCC)) {
                                coord++;
                                cp3(nd[j++], q);
                            }
                        }
                        if (j > 4) ora_fail(o, "SetSiCSF: more than four shell neighbours at %d %d %d", x, y, z);
                    }
                    if (pass == 0) {                /* :209-220 */
                        if (coord > coor) {
                            if (coord <= 1) *v = 0;
                        } else if (coor <= 1) {
                            *v = 0;
                        }
                        continue;
                    }
                    int ev;
                    double prob;
                    const int iat = ibits(*v, POS_SIC, LEN_SIC);
                    if (coord > coor) {             /* :284-317 */
                        mvbits(coord, LEN_COOR, v, POS_COOR);
                        int nn4[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                        for (int i = 0; i < j && i < 4; i++) cp3(nn4[i], nd[i]);
                        if (coord <= 3) {
                            int ns2[2][3];
                            find_nn(nn4[0], nn4[1], site, ns2, lx, ly);
                            cp3(nn4[2], ns2[0]);
                            cp3(nn4[3], ns2[1]);
                            get_prob_ini(o, 1, iat, coord, site, nn4, &ev, &prob);
                            add_mc(o, site, nn4, ev, prob);
                        } else {
                            add_bulk(o, site, nn4);
                        }
                    } else {                        /* :318-330 */
                        mvbits(coor, LEN_COOR, v, POS_COOR);
                        if (coor <= 3) {
                            get_prob_ini(o, 1, iat, coor, site, nextn, &ev, &prob);
                            add_mc(o, site, nextn, ev, prob);
                        } else {
                            add_bulk(o, site, nextn);
                        }
                    }
                }
    /* :336-377 (MC atoms) and :380-427 (bulk atoms of z >= 13): reciprocal bonds only */
    for (int kind = 0; kind < 2; kind++) {
        const int64_t n0 = kind == 0 ? o->num_mc : o->num_bulk;
        for (int64_t i = 1; i <= n0; i++) {
            int nn4[4][3];
            if (kind == 0) {
                cp3(site, o->mc[i].xyz);
                memcpy(nn4, o->mc[i].nn, sizeof nn4);
            } else {
                cp3(site, o->bulk[i].xyz);
                if (site[2] < 13) continue;
                memcpy(nn4, o->bulk[i].nn, sizeof nn4);
            }
            int32_t *v = LC(o, site);
            int coor = ibits(*v, POS_COOR, LEN_COOR);
            const int coor_old = coor;
            for (int jn = 0; jn < 4; jn++) {
                const int32_t w = *LC(o, nn4[jn]);
                if (!ibits(w, POS_OCC, LEN_OCC)) continue;
                const int ind_nn = *LI(o, nn4[jn]);
                const int(*back)[3] = ibits(w, POS_COOR, LEN_COOR) == 4 ? o->bulk[ind_nn].nn : o->mc[ind_nn].nn;
                int recip = 0;
                for (int kk = 0; kk < 4; kk++) recip |= same3(back[kk], site);
                if (!recip) coor--;
            }
            if (coor == coor_old) continue;
            const int inds = *LI(o, site);
            const int iat = ibits(*v, POS_SIC, LEN_SIC);
            mvbits(coor, LEN_COOR, v, POS_COOR);
            int ev;
            double prob;
            get_prob(o, 1, iat, 0, coor, site, nn4, &ev, &prob);
            if (kind == 0) {
                o->mc[inds].ind_event = ev;
                o->mc[inds].prob = prob;
                update_tree(o, inds, prob);
            } else {
                erase_bulk(o, site);
                add_mc(o, site, nn4, ev, prob);
            }
        }
    }
    /* :429-471: the ad-voids of every MC atom's NextN */
    const int nmc_old = o->num_mc;
    for (int i = 1; i <= nmc_old; i++) {
        int nns[3];
        cp3(nns, o->mc[i].xyz);
        for (int jn = 0; jn < 4; jn++) {
            cp3(site, o->mc[i].nn[jn]);
            int32_t *v = LC(o, site);
            if (ibits(*v, POS_OCC, LEN_OCC)) continue;
            int nn4[4][3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            const int coor = ibits(*v, POS_COOR, LEN_COOR) + 1;
            int ev;
            double prob;
            if (coor == 1) {
                cp3(nn4[0], nns);
                mvbits(coor, LEN_COOR, v, POS_COOR);
                get_prob_ini(o, 0, 0, coor, site, nn4, &ev, &prob);
                add_mc(o, site, nn4, ev, prob);
            } else if (coor == 2) {
                const int inds = *LI(o, site);
                memcpy(nn4, o->mc[inds].nn, sizeof nn4);
                cp3(nn4[1], nns);
                int ns2[2][3];
                find_nn(nn4[0], nn4[1], site, ns2, lx, ly);
                cp3(nn4[2], ns2[0]);
                cp3(nn4[3], ns2[1]);
                mvbits(coor, LEN_COOR, v, POS_COOR);
                get_prob_ini(o, 0, 0, coor, site, nn4, &ev, &prob);
                memcpy(o->mc[inds].nn, nn4, sizeof nn4);
                o->mc[inds].ind_event = ev;
                o->mc[inds].prob = prob;
                update_tree(o, inds, prob);
            } else if (coor == 3) {
                const int inds = *LI(o, site);
                memcpy(nn4, o->mc[inds].nn, sizeof nn4);
                mvbits(coor, LEN_COOR, v, POS_COOR);
                get_prob_ini(o, 0, 0, coor, site, nn4, &ev, &prob);
                o->mc[inds].ind_event = ev;
                o->mc[inds].prob = prob;
                update_tree(o, inds, prob);
            } else {
                ora_fail(o, "Vacancy in the SF setting");
            }
        }
    }
}

int ora_init(ora_t *o)
{
    if (setjmp(o->jb)) return -1;
    /* MS/main.f:224-295 */
    if (!strcmp(o->init_st, "FS")) {
        o->len1 -= o->len1 % 24;
        set_flat(o, o->len1, 0, 1);
    } else if (!strcmp(o->init_st, "Fw") || !strcmp(o->init_st, "Fa")) {   /* MS/main.f:228-236 */
        o->len1 -= o->len1 % 24;
        o->len2 -= o->len2 % 24;
        o->len3 -= o->len3 % 24;
        set_flat(o, o->len1, 1, 1);
        set_wall_block(o, o->len2, o->init_st[1] == 'a' ? o->len3 : -1);
    } else if (!strcmp(o->init_st, "FF")) {      /* MS/main.f:273-278 */
        o->len1 -= o->len1 % 24;
        o->len2 -= o->len2 % 24;
        o->len3 -= o->len3 % 24;
        o->len4 -= o->len4 % 24;
        set_finfet(o, o->len1, o->len2, o->len3, o->len4);
    } else if (!strcmp(o->init_st, "F")) {
        o->len1 -= o->len1 % 24;
        set_flat(o, o->len1, 1, 0);
    } else if (!strcmp(o->init_st, "C")) {       /* MS/main.f:261-262 */
        set_nc(o, o->len1, o->len2, o->len3, 0, 0);
    } else if (!strcmp(o->init_st, "S") || !strcmp(o->init_st, "SS")) {   /* MS/main.f:257-260 */
        set_nc(o, o->len1, o->len1, o->len1, 1, o->init_st[1] == 'S');
    } else if (!strcmp(o->init_st, "ST")) {      /* MS/main.f:265-266 */
        set_trench(o, o->len1, o->len2, o->len3, 0);
    } else if (!strcmp(o->init_st, "T")) {       /* MS/main.f:263-264 */
        set_trench(o, o->len1, o->len2, o->len3, 1);
    } else if (o->init_st[0] && strchr("IDZJKL", o->init_st[0]) && o->init_st[1] == 0) {   /* MS/main.f:245-256 */
        set_invp(o, o->len1, o->len2, o->init_st[0]);
    } else if (!strcmp(o->init_st, "LA")) {      /* MS/main.f:287-291 */
        if (!o->la_geo) ora_fail(o, "InitSt LA needs the geometry and temperature input (ora_set_la_input)");
        set_cad(o, 1);
    } else if (!strcmp(o->init_st, "IN")) {      /* MS/main.f:279-280 */
        if (!o->cad_geo) ora_fail(o, "InitSt IN needs the per-site geometry (ora_set_geometry)");
        if (o->ncrystal != 1) ora_fail(o, "the IN initializer is restated for NCrystal = 1");
        set_cad(o, 0);
    } else if (!strcmp(o->init_st, "SH")) {      /* MS/main.f:281-286 */
        set_shape(o);
    } else if (!strcmp(o->init_st, "E")) {       /* MS/main.f:267-272 */
        const int vsf[3] = {o->len2, o->len3, o->len1 - o->len2};
        lg(o, " %d %d %d %d\n", o->len1, vsf[0], vsf[1], vsf[2]);
        set_sicsf(o, o->len1, vsf);
    } else {
        ora_fail(o, "initialization not_implemented in the oracle: %s", o->init_st);
    }
    lg(o, " Atoms,Voids,AdAtoms %lld %d %d\n", (long long)o->num_bulk, o->num_void, o->num_mc);
    memcpy(o->count_crystal_old, o->count_crystal, sizeof o->count_crystal);
    return 0;
}

static void trace_push(ora_t *o, const int site[3], int itrans, int arm)
{
    if (!o->trace_on) return;
    if (o->trace_len >= o->trace_cap) {
        int64_t nc = o->trace_cap ? o->trace_cap * 2 : (1 << 16);
        ora_event_t *t = (ora_event_t *)realloc(o->trace, (size_t)nc * sizeof(ora_event_t));
        if (!t) ora_fail(o, "trace allocation failed");
        o->trace = t;
        o->trace_cap = nc;
    }
    ora_event_t *e = &o->trace[o->trace_len++];
    e->x = site[0]; e->y = site[1]; e->z = site[2];
    e->itrans = (int8_t)itrans;
    e->arm = (int8_t)arm;
    e->pad = 0;
}

/* One iteration of the KMC loop, MS/main.f:304-369.  Returns 1 to exit. */
static int kmc_step(ora_t *o, const char *outdir)
{
    o->iter_out = o->iter;
    if (o->num_mc <= 20) {
        lg(o, " few MC particles: stop MC %lld %d\n", (long long)o->iter, o->num_mc);
        return 1;
    }
    double patom;
    int ind = pick_tree_event(o, &patom);
    o->time = o->time + 1.0 / o->tree[1];
    int itrans = o->mc[ind].ind_event;
    if (!strcmp(o->exit_strategy, "Iter")) {
        if (o->out_molmol > 0 && o->iter % o->out_molmol == 0) {
            o->framecounter = o->iter_out / o->out_molmol;
            write_molmol_source(o, outdir, o->time, o->iter_out, o->framecounter);
            int *s = o->mc[ind].xyz;
            lg(o, " Iter, Time, Site %lld %.17g %d %d %d\n", (long long)o->iter, o->time, s[0], s[1], s[2]);
            lg(o, " NatNvoidNad %lld %d %d\n", (long long)o->num_bulk, o->num_void, o->num_mc);
        }
    } else if (!strcmp(o->exit_strategy, "Time")) {
        if (o->time >= (double)(o->framecounter + 1) * o->out_time) {
            write_molmol_source(o, outdir, o->time, o->iter_out, o->framecounter + 1);
            int *s = o->mc[ind].xyz;
            lg(o, " Iter, Time, Site %lld %.17g %d %d %d\n", (long long)o->iter, o->time, s[0], s[1], s[2]);
            lg(o, " NatNvoidNad %lld %d %d\n", (long long)o->num_bulk, o->num_void, o->num_mc);
            o->framecounter++;
        }
    }
    int site[3];
    cp3(site, o->mc[ind].xyz);
    if (itrans <= 3) {
        deposition(o, ind, itrans);
        if (itrans >= 1) o->count_crystal[itrans - 1]++;
        trace_push(o, site, itrans, o->cur_arm);
    } else if (itrans == 4) {
        evaporation(o, ind);
        trace_push(o, site, 4, 0);
    } else if (itrans == 5) {
        desorption(o, ind);
        trace_push(o, site, 5, 0);
    } else {
        int covind = o->list_cov[itrans - 6];
        absorption(o, ind, covind);
        o->count_cov[itrans - 6]++;
        trace_push(o, site, itrans, 0);
    }
    o->iter++;
    if (!strcmp(o->exit_strategy, "Iter")) {
        if (o->iter > o->max_iter) return 2;
    } else if (!strcmp(o->exit_strategy, "Time")) {
        if (o->time > o->max_time) return 2;
    }
    return 0;
}

int ora_run(ora_t *o, int64_t n, const char *outdir)
{
    if (setjmp(o->jb)) return -1;
    if (!o->started) {
        write_molmol_source(o, outdir, o->time, 0, 0);
        o->started = 1;
    }
    for (int64_t k = 0; k < n; k++) {
        int r = kmc_step(o, outdir);
        if (r) return r;
    }
    return 0;
}

int ora_run_until(ora_t *o, double tmax)
{
    if (setjmp(o->jb)) return -1;
    o->started = 1;
    while (o->time <= tmax) {
        int r = kmc_step(o, NULL);
        if (r) return r;
    }
    return 0;
}

int ora_main(ora_t *o, const char *outdir)
{
    o->log = stdout;
    if (ora_init(o)) return -1;
    if (setjmp(o->jb)) return -1;
    write_molmol_source(o, outdir, o->time, 0, 0);
    o->started = 1;
    for (;;) {
        int r = kmc_step(o, outdir);
        if (r < 0) return -1;
        if (r) break;
    }
    if (!strcmp(o->exit_strategy, "Iter"))
        write_molmol_source(o, outdir, o->time, o->iter_out, o->out_molmol > 0 ? o->iter_out / o->out_molmol : 0);
    else
        write_molmol_source(o, outdir, o->time, o->iter_out, o->framecounter);
    return 0;
}

void ora_trace_enable(ora_t *o, int on) { o->trace_on = on; }
int64_t ora_trace_len(const ora_t *o) { return o->trace_len; }
const ora_event_t *ora_trace(const ora_t *o) { return o->trace; }
void ora_trace_clear(ora_t *o) { o->trace_len = 0; }
int64_t ora_iter(const ora_t *o) { return o->iter; }
double ora_time(const ora_t *o) { return o->time; }
double ora_total_rate(const ora_t *o) { return o->tree[1]; }
int ora_counts(const ora_t *o, int32_t out[3])
{
    out[0] = (int32_t)o->num_bulk;
    out[1] = o->num_void;
    out[2] = o->num_mc;
    return 0;
}
void ora_dims(const ora_t *o, int32_t out[3])
{
    out[0] = o->lx; out[1] = o->ly; out[2] = o->lz;
}
void ora_get_lattcoo(const ora_t *o, int32_t *out)
{
    memcpy(out, o->latt, sizeof(int32_t) * (size_t)o->lx * o->ly * ((size_t)o->lz + 1));
}
int ora_site_info(const ora_t *o, int x, int y, int z, int32_t nn[12], int32_t *ind_event, double *prob)
{
    int64_t i = lidx(o, x, y, z);
    int32_t v = o->latt[i];
    int ind = o->lind[i];
    int occ = ibits(v, POS_OCC, LEN_OCC), coo = ibits(v, POS_COOR, LEN_COOR);
    int which = 0;
    if (ind == 0) which = 0;
    else if (occ == 1 && coo == 4) which = 2;
    else if (occ == 0 && coo == 4) which = 3;
    else which = 1;
    *ind_event = 0;
    *prob = 0.0;
    if (which == 1) {
        memcpy(nn, o->mc[ind].nn, sizeof(int32_t) * 12);
        *ind_event = o->mc[ind].ind_event;
        *prob = o->mc[ind].prob;
    } else if (which == 2) {
        memcpy(nn, o->bulk[ind].nn, sizeof(int32_t) * 12);
    } else if (which == 3) {
        memcpy(nn, o->voids[ind].nn, sizeof(int32_t) * 12);
    } else {
        memset(nn, 0, sizeof(int32_t) * 12);
    }
    return which;
}
int ora_write_xyz(ora_t *o, const char *path)
{
    if (setjmp(o->jb)) return -1;
    FILE *f = fopen(path, "w");
    if (!f) return -1;
    write_xyz_files(o, f, NULL, NULL, NULL, o->time, o->iter_out);
    fclose(f);
    return 0;
}
/* All four frame files of WriteMolMolXYZFile (<base>.xyz, _d, _v, _w) with
 * the given clock and iteration; for SiC the swap-and-restore of the wrong
 * sites is applied to the oracle's lattice, as the reference does. */
int ora_write_frame(ora_t *o, const char *base, double time, int64_t iter)
{
    if (setjmp(o->jb)) return -1;
    char p[4][2100];
    snprintf(p[0], sizeof p[0], "%s.xyz", base);
    snprintf(p[1], sizeof p[1], "%s_d.xyz", base);
    snprintf(p[2], sizeof p[2], "%s_v.xyz", base);
    snprintf(p[3], sizeof p[3], "%s_w.xyz", base);
    FILE *f[4];
    for (int i = 0; i < 4; i++) {
        f[i] = fopen(p[i], "w");
        if (!f[i]) {
            for (int j = 0; j < i; j++) fclose(f[j]);
            return -1;
        }
    }
    write_xyz_files(o, f[0], f[1], f[2], f[3], time, iter);
    for (int i = 0; i < 4; i++) fclose(f[i]);
    return 0;
}

void ora_get_rates(const ora_t *o, double ptransE[3 * 4096], double ptransD[9])
{
    int k = 0;
    for (int s = 0; s < 3; s++)
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++)
                for (int c = 0; c < 4; c++)
                    for (int d = 0; d < 4; d++)
                        for (int e = 0; e < 4; e++)
                            for (int f = 0; f < 4; f++) ptransE[k++] = o->ptransE[s][a][b][c][d][e][f];
    for (int s = 0; s < 3; s++)
        for (int c = 0; c < 3; c++) ptransD[s * 3 + c] = o->ptransD[s][c];
}

int ora_ncov(const ora_t *o) { return o->ncov; }

void ora_get_cov_rates(const ora_t *o, double ptransAbs[9], double ptransDes[9])
{   /* [coverage species][coor-1] */
    for (int s = 0; s < 3; s++)
        for (int c = 1; c <= 3; c++) {
            ptransAbs[s * 3 + c - 1] = o->ptransAbs[s][c];
            ptransDes[s * 3 + c - 1] = o->ptransDes[s][c];
        }
}

/* Conversion to the one-byte-per-site layout of the GPU engine (used by the
 * parity tests to compare states). */
int64_t ora_compact_state(const ora_t *o, uint8_t *out)
{
    static const int OFF[2][4][3] = {{{0, 0, 1}, {0, -1, -1}, {-1, -1, 1}, {-1, 0, -1}},
                                     {{1, 1, -1}, {1, 0, 1}, {0, 0, -1}, {0, 1, 1}}};
    int na = o->lx / 6, nb = o->ly / 6, nz = o->lz / 3 + 1;
    int64_t offgrid = 0;
    for (int z = 0; z <= o->lz; z++)
        for (int y = 0; y < o->ly; y++)
            for (int x = 0; x < o->lx; x++) {
                int32_t v = o->latt[lidx(o, x, y, z)];
                if (v && ibits(v, POS_INDEX, LEN_INDEX) != WALL && !dia_kind(x, y, z)) offgrid++;
            }
    for (int z1 = 0; z1 < nz; z1++)
        for (int b = 0; b < nb; b++)
            for (int a = 0; a < na; a++) {
                uint8_t *d = &out[((size_t)z1 * nb + b) * na + a];
                *d = 0;
                if ((a + b + (z1 >> 1)) & 1) continue;
                int x = 3 * (2 * a + (z1 & 1)), y = 3 * (2 * b + (z1 & 1)), z = 3 * z1;
                int32_t v = o->latt[lidx(o, x, y, z)];
                if (ibits(v, POS_INDEX, LEN_INDEX) == WALL) { *d = 0x80; continue; }
                if (!v) continue;
                int occ = ibits(v, POS_OCC, LEN_OCC), co = ibits(v, POS_COOR, LEN_COOR), sp = ibits(v, POS_SIC, LEN_SIC);
                int32_t nn[12], ie;
                double pr;
                int which = ora_site_info(o, x, y, z, nn, &ie, &pr);
                int fd = 0;
                if (which) {
                    fd = -1;
                    for (int dd = 0; dd < 4; dd++) {
                        int aa = ((a + OFF[z1 & 1][dd][0]) % na + na) % na;
                        int bb = ((b + OFF[z1 & 1][dd][1]) % nb + nb) % nb;
                        int kk = z1 + OFF[z1 & 1][dd][2];
                        if (3 * (2 * aa + (kk & 1)) == nn[0] && 3 * (2 * bb + (kk & 1)) == nn[1] && 3 * kk == nn[2]) fd = dd;
                    }
                    if (fd < 0) return -1;
                }
                /* the dummy rate of Get_Prob (1e-8) is the flag; that of
                 * Get_Prob_Ini (1e-6) the flag with coordination field 5 */
                int dm = (!occ && co == 1 && which == 1 && (pr == (double)1.e-8f || pr == (double)1.e-6f)) ? 1 : 0;
                if (dm && pr == (double)1.e-6f) co = 5;
                /* an empty site carrying a coverage species is species value
                 * 3, with bit 7 set for the second coverage species */
                if (!occ && ibits(v, POS_INDEX, LEN_INDEX) != 0) {
                    sp = 3;
                    dm = (o->ncov >= 2 && ibits(v, POS_INDEX, LEN_INDEX) == o->list_cov[1]) ? 1 : 0;
                }
                *d = (uint8_t)((sp & 3) | ((co & 7) << 2) | (fd << 5) | (dm << 7));
            }
    return offgrid;
}

/* census enumeration shared with the GPU engine: (n1,n2,n3) with
 * 1 <= n1+n2+n3 <= 3, by total, then n1 descending, then n2 descending */
static int census_idx(int n1, int n2, int n3)
{
    int k = 0;
    for (int t = 1; t <= 3; t++)
        for (int a = t; a >= 0; a--)
            for (int b = t - a; b >= 0; b--) {
                int c = t - a - b;
                if (a == n1 && b == n2 && c == n3) return k;
                k++;
            }
    return -1;
}

/* Grid coordinates of the MC particles in list order (ListAdAtom(i) %
 * AtomXYZ, defdertype.f:32-37), up to n of them; returns NumAdAtom. */
int64_t ora_mc_sites(const ora_t *o, int32_t *xyz, int64_t n)
{
    for (int i = 1; i <= o->num_mc && i <= n; i++)
        for (int k = 0; k < 3; k++) xyz[3 * (i - 1) + k] = o->mc[i].xyz[k];
    return o->num_mc;
}

/* Every list entry: the MC particles (kind 1, ListAdAtom), the bulk atoms
 * (kind 2, ListAtom) and the voids (kind 3, ListVoid), each list in its
 * order, with the grid point, the four NextN entries, and for MC particles
 * Ind_Event and ProbTrans (defdertype.f:25-45).  Writes up to n entries;
 * returns the total count. */
int64_t ora_list_entries(const ora_t *o, int32_t *xyz, int32_t *nn, int32_t *kind, int32_t *ind_event,
                         double *prob, int64_t n)
{
    int64_t k = 0;
    for (int pass = 1; pass <= 3; pass++) {
        int64_t m = pass == 1 ? o->num_mc : (pass == 2 ? o->num_bulk : o->num_void);
        for (int64_t i = 1; i <= m; i++, k++) {
            if (k >= n) continue;
            const int *p = pass == 1 ? o->mc[i].xyz : (pass == 2 ? o->bulk[i].xyz : o->voids[i].xyz);
            const int(*q)[3] = pass == 1 ? o->mc[i].nn : (pass == 2 ? o->bulk[i].nn : o->voids[i].nn);
            for (int c = 0; c < 3; c++) xyz[3 * k + c] = p[c];
            for (int j = 0; j < 4; j++)
                for (int c = 0; c < 3; c++) nn[12 * k + 3 * j + c] = q[j][c];
            kind[k] = pass;
            ind_event[k] = pass == 1 ? o->mc[i].ind_event : 0;
            prob[k] = pass == 1 ? o->mc[i].prob : 0.0;
        }
    }
    return k;
}

int64_t ora_mc_classes(const ora_t *o_, int32_t *cls, double *rate, int64_t n)
{
    ora_t *o = (ora_t *)o_;
    for (int i = 1; i <= o->num_mc && i <= n; i++) {
        mcp_t *p = &o->mc[i];
        int32_t v = *LC(o, p->xyz);
        int occ = ibits(v, POS_OCC, LEN_OCC), co = ibits(v, POS_COOR, LEN_COOR);
        int sp = ibits(v, POS_SIC, LEN_SIC);
        int c = 0;
        if (!occ && o->ncov > 0 && ibits(v, POS_INDEX, LEN_INDEX) != 0) {
            /* covered: desorption, 6..8 for ListCov(1), 59..61 for ListCov(2) */
            int second = o->ncov >= 2 && ibits(v, POS_INDEX, LEN_INDEX) == o->list_cov[1];
            if (co >= 1 && co <= 3) c = (second ? 59 : 6) + co - 1;
        } else if (!occ) {
            if (co == 1) c = (p->prob == (double)1.e-8f) ? 2 : (p->prob == (double)1.e-6f ? 63 : 1);
            else if (co == 2) c = 3;
            else if (co == 3) c = 4;
        } else if (o->ncov > 0) {
            /* census (nSi+nWall, nC) and covered neighbours as Get_Prob.f:
             * 215-291 counts them, reciprocity through each neighbour's list */
            int n_si = 0, n_c = 0, n_w = 0, n_cov = 0, n_cov2 = 0;
            for (int k = 0; k < 4; k++) {
                int32_t w = *LC(o, p->nn[k]);
                int cn = ibits(w, POS_COOR, LEN_COOR), ind = *LI(o, p->nn[k]);
                int nnn[4][3];
                if (!ibits(w, POS_OCC, LEN_OCC)) {
                    if (ibits(w, POS_INDEX, LEN_INDEX) == 0) continue;
                    get_nn_list(o, ind, 1, nnn);
                    if (in_list(nnn, p->xyz)) {
                        if (o->ncov >= 2 && ibits(w, POS_INDEX, LEN_INDEX) == o->list_cov[1]) n_cov2++;
                        else n_cov++;
                    }
                    continue;
                }
                if (ibits(w, POS_INDEX, LEN_INDEX) == WALL) { n_w++; continue; }
                get_nn_list(o, ind, (cn >= 1 && cn <= 3) ? 1 : 2, nnn);
                if (!in_list(nnn, p->xyz)) continue;
                int s2 = ibits(w, POS_SIC, LEN_SIC);
                if (s2 == 1) n_si++;
                if (s2 == 2) n_c++;
            }
            int t = n_si + n_c + n_w;
            if (t == 0) c = 5;
            else if (t <= 3 && o->ncov >= 2) {
                /* (n1, c1, c2), c1 + c2 <= 4 - n1: 19 classes from 9 */
                int n1 = n_si + n_w, m = 4 - n1, base = n1 == 1 ? 0 : (n1 == 2 ? 10 : 16);
                c = 9 + base + n_cov * (m + 1) - n_cov * (n_cov - 1) / 2 + n_cov2;
            } else if (t <= 3) {
                int n1 = n_si + n_w, base = t == 1 ? 0 : (t == 2 ? 8 : 17);
                c = 9 + (sp - 1) * 25 + base + (t - n1) * (5 - t) + n_cov;
            }
        } else {
            int n_si = 0, n_c = 0, n_b = 0, n_w = 0;
            for (int k = 0; k < 4; k++) {
                int32_t w = *LC(o, p->nn[k]);
                if (!ibits(w, POS_OCC, LEN_OCC)) continue;
                if (ibits(w, POS_INDEX, LEN_INDEX) == WALL) { n_w++; continue; }
                int cn = ibits(w, POS_COOR, LEN_COOR);
                int ind = *LI(o, p->nn[k]);
                int nnn[4][3];
                get_nn_list(o, ind, (cn >= 1 && cn <= 3) ? 1 : 2, nnn);
                if (!in_list(nnn, p->xyz)) continue;
                int s2 = ibits(w, POS_SIC, LEN_SIC);
                if (s2 == 1) n_si++;
                if (s2 == 2) n_c++;
                if (s2 == 3) n_b++;
            }
            int t = n_si + n_c + n_b + n_w;
            if (t == 0) c = 5;
            else if (t <= 3) c = 6 + (sp - 1) * 19 + census_idx(n_si + n_w, n_c, n_b);
        }
        cls[i - 1] = c;
        rate[i - 1] = p->prob;
    }
    return o->num_mc;
}

/* ============ per-species LA law, liquid fractions and LR score ============
 * The LaserAnnealing variant's rate law (LA/mcevent/Get_Prob.f:127-152,
 * per-species P0, Tm, Tflex, sigma; solidification weighted by the liquid
 * fraction CountLiquid/SUM(CountLiquid) with CountLiquid = InitCountCrystal -
 * CountCrystal, LA/main.f:637, Evaporation.f:41, main.f:683) on the lists and
 * event routines above, with a prescribed temperature field.  The clock is a
 * continuous-time Markov chain with exponential waiting times and every rate
 * recomputed from the lattice before each draw (a linear scan instead of the
 * sum tree), so that the likelihood-ratio score
 *     S_j = sum_events d log k / d theta_j - int sum_sites d k / d theta_j dt
 * is exact; it is accumulated in FP64.  Time is cut into windows of length
 * tau: the temperature of a window is taken at its midpoint, the liquid
 * fractions are refreshed every `phase` windows and the stop rules (more atoms
 * than at the start, LA/main.f:714-723; <= 20 MC particles, main.f:307-310)
 * are checked at window ends — the schedule of the GPU engine's LA mode.
 * A SiGe solidification of a species whose crystal count has reached its
 * initial count deposits the other species instead (LA/main.f:676-681).   */

static uint64_t la_next(ora_t *o)
{   /* xoshiro256** (Blackman & Vigna) */
    uint64_t *q = o->la_rng;
    uint64_t r = q[1] * 5;
    r = ((r << 7) | (r >> 57)) * 9;
    uint64_t t = q[1] << 17;
    q[2] ^= q[0]; q[3] ^= q[1]; q[1] ^= q[2]; q[0] ^= q[3];
    q[2] ^= t;
    q[3] = (q[3] << 45) | (q[3] >> 19);
    return r;
}
static double la_u01(ora_t *o) { return ((double)(la_next(o) >> 11) + 0.5) * (1.0 / 9007199254740992.0); }

/* reciprocal occupied neighbours by species (walls count as species 1), as
 * the occupied branch of get_prob (Get_Prob.f:230-300) */
static int la2_census(ora_t *o, const int site[3], int nextn[4][3], int *n1, int *n2, int *n3)
{
    int n_si = 0, n_c = 0, n_b = 0, n_wall = 0;
    for (int i = 0; i < 4; i++) {
        int32_t v = *LC(o, nextn[i]);
        if (ibits(v, POS_OCC, LEN_OCC) == 0) continue;
        if (ibits(v, POS_INDEX, LEN_INDEX) == WALL) { n_wall++; continue; }
        int coornn = ibits(v, POS_COOR, LEN_COOR);
        int nnn[4][3];
        get_nn_list(o, *LI(o, nextn[i]), (coornn >= 1 && coornn <= 3) ? 1 : 2, nnn);
        if (!in_list(nnn, site)) continue;
        int sp = ibits(v, POS_SIC, LEN_SIC);
        if (sp == 1) n_si++;
        if (sp == 2) n_c++;
        if (sp == 3) n_b++;
    }
    *n1 = n_si + n_wall; *n2 = n_c; *n3 = n_b;
    return n_si + n_c + n_b + n_wall;
}

enum { LK_NONE = 0, LK_DEP = 1, LK_DUMMY = 2, LK_MELT = 3, LK_ISO = 4 };

/* rate k of MC particle ind, dk/dtheta, and per-species solidification rates */
static int la2_rate(ora_t *o, int ind, double *k, double dk[4], double ps[3])
{
    mcp_t *m = &o->mc[ind];
    int32_t v = *LC(o, m->xyz);
    int occ = ibits(v, POS_OCC, LEN_OCC), coor = ibits(v, POS_COOR, LEN_COOR);
    int T = la2_temp(o, m->xyz[2]);
    *k = 0.0;
    for (int j = 0; j < 4; j++) dk[j] = 0.0;
    ps[0] = ps[1] = ps[2] = 0.0;
    if (occ) {
        int n1, n2, n3, sp = ibits(v, POS_SIC, LEN_SIC);
        int tot = la2_census(o, m->xyz, m->nn, &n1, &n2, &n3);
        if (tot > 3 || sp < 1) return LK_NONE;
        if (tot == 0) return LK_ISO;
        double E = o->ptransE[sp - 1][n1][n2][n3][0][0][0];
        if (E == 0.0) return LK_NONE;
        *k = o->lap.P0[sp - 1] * exp(-E / (KB * (double)T));
        for (int j = 0; j < 4; j++) dk[j] = -*k * o->dE[sp - 1][n1][n2][n3][j] / (KB * (double)T);
        return LK_MELT;
    }
    if (coor == 1 && m->prob == (double)1.e-8f) {   /* Get_Prob.f:181-184 */
        *k = (double)1.e-8f;
        return LK_DUMMY;
    }
    if (coor < 1 || coor > 3) return LK_NONE;
    o->la_cur_z = m->xyz[2];
    for (int s = 0; s < 3; s++) {
        ps[s] = la2_pd(o, s + 1, coor, T);
        *k += ps[s];
        for (int j = 0; j < 4; j++) dk[j] -= ps[s] * o->dEd[s][coor - 1][j] / (KB * o->lap.Tm[s]);
    }
    return LK_DEP;
}

static void la2_refresh_xliq(ora_t *o)
{
    int64_t liq[3], sum = 0;
    for (int s = 0; s < 3; s++) {
        liq[s] = o->la_init[s] - o->la_cnt[s];
        if (liq[s] < 0) liq[s] = 0;
        sum += liq[s];
    }
    for (int s = 0; s < 3; s++) o->xliq[s] = sum > 0 ? (double)liq[s] / (double)sum : 0.0;
}

static int64_t la2_species_count(ora_t *o, int64_t out[3])
{
    out[0] = out[1] = out[2] = 0;
    for (int z = 0; z <= o->lz; z++)
        for (int y = 0; y < o->ly; y++)
            for (int x = 0; x < o->lx; x++) {
                int32_t v = o->latt[lidx(o, x, y, z)];
                if (!ibits(v, POS_OCC, LEN_OCC) || ibits(v, POS_INDEX, LEN_INDEX) == WALL) continue;
                int sp = ibits(v, POS_SIC, LEN_SIC);
                if (sp >= 1 && sp <= 3) out[sp - 1]++;
            }
    return out[0] + out[1] + out[2];
}

int ora_la_alloy(ora_t *o, double x, uint64_t seed)
{
    if (setjmp(o->jb)) return -1;
    uint64_t z = seed + 0x9E3779B97F4A7C15ull;
    for (int i = 0; i < 4; i++) {   /* splitmix64 */
        z += 0x9E3779B97F4A7C15ull;
        uint64_t r = z;
        r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ull;
        r = (r ^ (r >> 27)) * 0x94D049BB133111EBull;
        o->la_rng[i] = r ^ (r >> 31);
    }
    for (int zz = 0; zz <= o->lz; zz++)
        for (int y = 0; y < o->ly; y++)
            for (int xx = 0; xx < o->lx; xx++) {
                int32_t *v = &o->latt[lidx(o, xx, y, zz)];
                if (!ibits(*v, POS_OCC, LEN_OCC) || ibits(*v, POS_INDEX, LEN_INDEX) == WALL) continue;
                if (la_u01(o) < x) mvbits(2, LEN_SIC, v, POS_SIC);
            }
    return 0;
}

int ora_la_set(ora_t *o, const ora_la_t *p, const double *ptransE, const double *dptransE,
               const double *ptransD, const double *dptransD, uint64_t seed)
{
    if (setjmp(o->jb)) return -1;
    if (o->ncov != 0) ora_fail(o, "LA mode with coverage species is not restated");
    if (!(p->tau > 0.0) || p->phase < 1) ora_fail(o, "LA mode needs tau > 0 and phase >= 1");
    o->lap = *p;
    memset(o->ptransE, 0, sizeof o->ptransE);
    memset(o->dE, 0, sizeof o->dE);
    for (int s = 0; s < 3; s++)
        for (int a = 0; a < 4; a++)
            for (int b = 0; b < 4; b++)
                for (int c = 0; c < 4; c++) {
                    size_t k = (size_t)s * 4096 + a * 1024 + b * 256 + c * 64;
                    o->ptransE[s][a][b][c][0][0][0] = ptransE[k];
                    for (int j = 0; j < 4; j++) o->dE[s][a][b][c][j] = dptransE ? dptransE[k * 4 + j] : 0.0;
                }
    for (int s = 0; s < 3; s++)
        for (int n = 0; n < 3; n++) {
            o->ptransD[s][n] = ptransD[s * 3 + n];
            for (int j = 0; j < 4; j++) o->dEd[s][n][j] = dptransD ? dptransD[(s * 3 + n) * 4 + j] : 0.0;
        }
    uint64_t z = seed;
    for (int i = 0; i < 4; i++) {   /* splitmix64 */
        z += 0x9E3779B97F4A7C15ull;
        uint64_t r = z;
        r = (r ^ (r >> 30)) * 0xBF58476D1CE4E5B9ull;
        r = (r ^ (r >> 27)) * 0x94D049BB133111EBull;
        o->la_rng[i] = r ^ (r >> 31);
    }
    la2_species_count(o, o->la_init);
    memcpy(o->la_cnt, o->la_init, sizeof o->la_init);
    o->xliq[0] = o->xliq[1] = o->xliq[2] = 0.0;
    o->la_win = (int64_t)floor(o->time / p->tau + 0.5);
    o->time = (double)o->la_win * p->tau;
    o->la_events = 0;
    o->la_stop = 0;
    memset(o->la_score, 0, sizeof o->la_score);
    o->la2 = 1;
    o->started = 1;
    return 0;
}

int ora_la_run_until(ora_t *o, double t_end)
{
    if (setjmp(o->jb)) return -1;
    if (!o->la2) ora_fail(o, "LA mode is not set (ora_la_set)");
    const double tau = o->lap.tau;
    int nz = o->lz + 1;
    int *tprof = (int *)malloc(sizeof(int) * (size_t)nz);
    if (!tprof) ora_fail(o, "allocation failed");
    for (int z = 0; z < nz; z++) tprof[z] = la2_temp(o, z);
    int dirty = 1, niso = 0;
    double R = 0.0, Rrest = 0.0, G[4] = {0.0, 0.0, 0.0, 0.0};
    while (!o->la_stop && o->time < t_end - 0.5 * tau) {
        double wend = (double)(o->la_win + 1) * tau;
        if (dirty) {
            if (o->la_cap < o->num_mc + 2) {
                o->la_cap = 2 * (o->num_mc + 2);
                o->la_k = (double *)realloc(o->la_k, sizeof(double) * (size_t)o->la_cap);
                o->la_dk = (double *)realloc(o->la_dk, sizeof(double) * 4 * (size_t)o->la_cap);
                o->la_ps = (double *)realloc(o->la_ps, sizeof(double) * 3 * (size_t)o->la_cap);
                o->la_kind = (int *)realloc(o->la_kind, sizeof(int) * (size_t)o->la_cap);
                if (!o->la_k || !o->la_dk || !o->la_ps || !o->la_kind) {
                    free(tprof);
                    ora_fail(o, "allocation failed");
                }
            }
            Rrest = 0.0;
            niso = 0;
            for (int j = 0; j < 4; j++) G[j] = 0.0;
            for (int ind = 1; ind <= o->num_mc; ind++) {
                int kind = la2_rate(o, ind, &o->la_k[ind], &o->la_dk[4 * ind], &o->la_ps[3 * ind]);
                o->la_kind[ind] = kind;
                if (kind == LK_ISO) niso++;
                Rrest += o->la_k[ind];
                for (int j = 0; j < 4; j++) G[j] += o->la_dk[4 * ind + j];
            }
            R = Rrest * (1.0 + 1.0e5 * niso);   /* isolated atoms: 1e5 x total, Get_Prob.f:305 */
            dirty = 0;
        }
        double dt = R > 0.0 ? -log(la_u01(o)) / R : INFINITY;
        if (o->time + dt >= wend) {
            for (int j = 0; j < 4; j++) o->la_score[j] -= G[j] * (wend - o->time);
            o->time = wend;
            o->la_win++;
            if (o->la_win % o->lap.phase == 0) {
                double x0[3];
                memcpy(x0, o->xliq, sizeof x0);
                la2_refresh_xliq(o);
                if (memcmp(x0, o->xliq, sizeof x0)) dirty = 1;
            }
            int64_t crys = o->la_cnt[0] + o->la_cnt[1] + o->la_cnt[2];
            int64_t init = o->la_init[0] + o->la_init[1] + o->la_init[2];
            if (crys > init) o->la_stop = 4;
            else if (o->num_mc <= 20) o->la_stop = 1;
            for (int z = 0; z < nz; z++) {
                int t = la2_temp(o, z);
                if (t != tprof[z]) { tprof[z] = t; dirty = 1; }
            }
            continue;
        }
        o->time += dt;
        for (int j = 0; j < 4; j++) o->la_score[j] -= G[j] * dt;
        double target = la_u01(o) * R, acc = 0.0;
        int ind = 0;
        for (int i = 1; i <= o->num_mc; i++) {
            acc += o->la_kind[i] == LK_ISO ? 1.0e5 * Rrest : o->la_k[i];
            if (acc > target) { ind = i; break; }
        }
        if (ind == 0)   /* rounding at the top end: the last particle with a rate */
            for (int i = o->num_mc; i >= 1 && !ind; i--)
                if (o->la_kind[i] == LK_ISO || o->la_k[i] > 0.0) ind = i;
        if (ind == 0) break;
        mcp_t *m = &o->mc[ind];
        int site[3];
        cp3(site, m->xyz);
        int kind = o->la_kind[ind];
        int32_t v = *LC(o, site);
        int sp = ibits(v, POS_SIC, LEN_SIC), coor = ibits(v, POS_COOR, LEN_COOR);
        if (kind == LK_DEP) {
            const double *ps = &o->la_ps[3 * ind];
            double u = la_u01(o) * (ps[0] + ps[1] + ps[2]);
            int s = u < ps[0] ? 0 : (u < ps[0] + ps[1] ? 1 : 2);
            for (int j = 0; j < 4; j++) o->la_score[j] -= o->dEd[s][coor - 1][j] / (KB * o->lap.Tm[s]);
            /* LA/main.f:676-681: a SiGe deposition of a species whose crystal
             * count has reached its initial count deposits the other one */
            if (o->ncrystal == 2 && o->list_crystal[0] == 14 && o->list_crystal[1] == 32 && s < 2 &&
                o->la_cnt[s] >= o->la_init[s])
                s = 1 - s;
            deposition(o, ind, s + 1);
            o->la_cnt[s]++;
            o->count_crystal[s]++;
        } else if (kind == LK_DUMMY) {
            deposition(o, ind, 1);
            o->la_cnt[0]++;
            o->count_crystal[0]++;
        } else if (kind == LK_MELT) {
            int n1, n2, n3;
            la2_census(o, site, m->nn, &n1, &n2, &n3);
            int T = la2_temp(o, site[2]);
            for (int j = 0; j < 4; j++) o->la_score[j] -= o->dE[sp - 1][n1][n2][n3][j] / (KB * (double)T);
            evaporation(o, ind);
            o->la_cnt[sp - 1]--;
        } else if (kind == LK_ISO) {
            evaporation(o, ind);
            o->la_cnt[sp - 1]--;
        } else {
            free(tprof);
            ora_fail(o, "picked a particle without an event");
        }
        o->la_events++;
        o->iter++;
        dirty = 1;
    }
    free(tprof);
    return o->la_stop;
}

void ora_la_state(const ora_t *o, double score[4], int64_t crystal[3], double xliq[3], int64_t *events)
{
    for (int j = 0; j < 4; j++) score[j] = o->la_score[j];
    for (int s = 0; s < 3; s++) {
        crystal[s] = o->la_cnt[s];
        xliq[s] = o->xliq[s];
    }
    *events = o->la_events;
}
