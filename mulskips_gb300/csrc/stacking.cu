// stacking.cu — the MulSKIPS KMC with arm-chair (hexagonal) stacking on
// GB300 (sm_103a): the reference's explicit-neighbour data model on the
// device, advanced by the synchronous-sublattice method.
//
// Layout in HBM (one replica):
//   coo[z+ZG][y][x]  uint32 LattCoo word of every grid point (defsystem.f:
//                    87-91: bits 0-7 CovInd, 113 a wall; 23 Occ; 24-26 Coor;
//                    27-29 species), z from -ZG to lz+ZG (zero guard planes)
//   ind[z+ZG][y][x]  int32 record of the site (LattInd), 0 for none
//   rec[1..]         one 36-byte record per listed site: grid point, the four
//                    NextN coordinates (int16; defdertype.f:25-45), event
//                    code and FP32 rate; rec[0] stays zero, the reference's
//                    zero guard entry of every list
// The (x, y) plane is cut into an even number of square tiles per side, at
// least 24 grid units wide, coloured by tile parity (four colours).  An event
// writes its site and its NextN sites (one bond, <= 6 units after rounding)
// and reads two bonds away at most (<= 12 units): two tiles of one colour are
// a tile apart, so one tile's writes never meet another's reads.  In a window
// of length tau the four colours run in turn, each tile from the window's
// start to its end with exponential waiting times, one warp per tile:
// lanes sum the rates of the tile's list and find the drawn entry with a
// prefix scan, lane 0 applies the event (Deposition.f / Evaporation.f,
// serial by nature: every step reads what the previous one wrote).
// Each tile keeps a list of record ids with an event and, beside it, their
// rates (contiguous floats for the selection scans; every rate change writes
// the record's list slot).  An event of tile A may give a site of an idle
// neighbour tile B its event; B's list then grows by an atomic append.  At
// the start of its phase a tile compacts its list once a quarter of its
// entries are dead.
// Records freed by a tile wait on its pending stack until its next phase, so
// a record never changes its site while a list entry of the running phase
// could still select it.
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>
#include <string.h>
#include <math.h>
#include <vector>
#include <algorithm>
#include "stacking.cuh"
#include "rng.cuh"

namespace mks_stk {
namespace {

using mks::U4;
using mks::philox4x32_10;
using mks::u01;

constexpr int ZG = 8;               // guard planes below z = 0 and above z = lz
constexpr uint32_t B_OCC = 1u << 23;
constexpr int WALLIND = 113;        // CovInd of a wall (SetSi.f:38-46)
constexpr int TWMIN = 24;           // smallest tile side (grid units)
constexpr int LCAP = 4096;          // list entries per tile
constexpr int FCAP = 1024;          // free records per tile and stack
constexpr int ICAP = 1024;          // inbox entries per tile (sites given an event by a neighbour tile)
enum : uint8_t { EV_NONE = 0, EV_DEP = 1, EV_DUMMY = 2, EV_EVAP = 4, EV_ISO = 5 };
// F_LISTED: in its tile's list (slot valid unless F_PEND / F_INBOX);
// F_PEND: appended to the running tile's list at the end of the event;
// F_INBOX: waiting in its tile's inbox for the tile's next phase
enum : uint8_t { F_LISTED = 1, F_PEND = 2, F_INBOX = 4 };
// device error codes (err[0]); err[1..3] say where
enum { E_INVARIANT = 3, E_CAPACITY = 4, E_TIMEOUT = 6, E_NOTAPPLICABLE = 7, E_BOUNDS = 8, E_NBUFF = 9, E_ARM = 10 };

struct Rec {
    int16_t x, y, z;
    int16_t nn[4][3];
    uint8_t ev, flags;
    float rate;
    int32_t slot;          // position in its tile's list while F_LISTED
};
static_assert(sizeof(Rec) == 40, "record layout");

struct P3 {
    int x, y, z;
};

struct Dev {
    uint32_t *coo;
    int32_t *ind;
    Rec *rec;
    int lx, ly, lz;
    int tw, ntx, nty;
    int32_t *tl, *tl_n;        // tile lists [tile][LCAP] and their lengths
    int32_t *ib, *ib_n;        // tile inboxes [tile][ICAP] and their lengths
    float *tr;                 // the listed sites' rates beside tl: > 0 a rate, -1 an isolated atom, 0 none
    int32_t *fr, *fr_n;        // reusable records per tile [tile][FCAP]
    int32_t *fp, *fp_n;        // records freed in the tile's current phase
    int32_t *top;              // records handed out so far (+1: rec[0] is the guard)
    int rcap;
    int32_t *err;              // [0] first error code, [1..3] where
    int32_t *nmc;              // sites with an event (NumAdAtom)
    unsigned long long *events;
    int32_t *stop;             // set when fewer than 21 sites keep an event
    unsigned *windows_done;    // windows completed by the persistent kernel
    const double *pe;          // [3][4][4][4]: PTransE(s, n1, n2, n3, 0, 0, 0)
    const double *pd;          // [3][3]: PTransD(s, coor)
    const float *pef;          // the same PTransE entries in FP32
    const float *pds;          // [3] FP32 of the FP64 sum of PTransD(s, coor) over s; [3..8] species shares
    double cth[2], sth[2];     // FIND_NN: cos, sin of 2 pi irot / 3 (pi in single precision)
    double shift;              // FIND_SN: arm-chair shift 8.6602254037 (single precision)
    double pzig;               // PtransZig
    uint32_t k0, k1;           // seed
};

// Per-warp event context (lane 0).
struct Ctx {
    int tile;                  // running tile; -1 in the replay kernel
    P3 nbuff;                  // Evaporation.f's NBuff, kept across calls as there
    int forced_arm;            // replay: the trace's stacking choice
    uint32_t key2, key3;       // Philox counter words of the stacking ties
    uint32_t nties;
    int dmc;                   // change of the count of sites with an event
    int npend;                 // records of the running tile to append after this event
    int pend[4];
};

__device__ __forceinline__ int coor_of(uint32_t v) { return (v >> 24) & 7; }
__device__ __forceinline__ int occ_of(uint32_t v) { return (v >> 23) & 1; }
__device__ __forceinline__ int cov_of(uint32_t v) { return v & 255; }
__device__ __forceinline__ int sp_of(uint32_t v) { return (v >> 27) & 7; }
__device__ __forceinline__ uint32_t with_coor(uint32_t v, int c) { return (v & ~(7u << 24)) | ((uint32_t)(c & 7) << 24); }
__device__ __forceinline__ bool same(P3 a, P3 b) { return a.x == b.x && a.y == b.y && a.z == b.z; }
__device__ __forceinline__ int isign(int a, int b) { return b >= 0 ? abs(a) : -abs(a); }
// NINT: nearest integer, halves away from zero
__device__ __forceinline__ int nint(double v) { return (int)round(v); }

// Set by set_err for the block that raised an error: the window kernel's
// warps test it after each event (a shared-memory read) instead of reading
// the grid's error word from L2; errors of other blocks stop them at the
// next grid barrier.  Kernels that do not read it leave it unset.
__shared__ int s_block_err;

__device__ void set_err(const Dev &D, int code, int a = 0, int b = 0, int c = 0)
{
    s_block_err = 1;
    if (atomicCAS(D.err, 0, code) == 0) {
        D.err[1] = a;
        D.err[2] = b;
        D.err[3] = c;
    }
}

// grid point -> array index; a point outside the arrays is an error and
// reads (0, 0, 0) instead, so no access leaves the arrays
__device__ __forceinline__ bool block_err() { return *(volatile int *)&s_block_err != 0; }

__device__ __forceinline__ int64_t gidx(const Dev &D, P3 p)
{
    if (p.x < 0 || p.x >= D.lx || p.y < 0 || p.y >= D.ly || p.z < -ZG || p.z > D.lz + ZG) {
        set_err(D, E_BOUNDS, p.x, p.y, p.z);
        return (int64_t)ZG * D.ly * D.lx;
    }
    return ((int64_t)(p.z + ZG) * D.ly + p.y) * D.lx + p.x;
}
__device__ __forceinline__ uint32_t cw(const Dev &D, P3 p) { return D.coo[gidx(D, p)]; }
__device__ __forceinline__ int tile_of(const Dev &D, int x, int y) { return (y / D.tw) * D.ntx + x / D.tw; }
__device__ __forceinline__ P3 nn_at(const Rec &r, int i) { return P3{r.nn[i][0], r.nn[i][1], r.nn[i][2]}; }
__device__ __forceinline__ void put_nn(Rec &r, int i, P3 p)
{
    r.nn[i][0] = (int16_t)p.x;
    r.nn[i][1] = (int16_t)p.y;
    r.nn[i][2] = (int16_t)p.z;
}
__device__ __forceinline__ bool in_list(const P3 nn[4], P3 s)
{
    return same(nn[0], s) || same(nn[1], s) || same(nn[2], s) || same(nn[3], s);
}
__device__ __forceinline__ void load_nn(const Rec &r, P3 nn[4])
{
    for (int i = 0; i < 4; i++) nn[i] = nn_at(r, i);
}
// The first 32 bytes of record r (x, y, z, the NextN list, ev, flags) as
// four 8-byte words: the pool is 256-byte aligned and records sit at 40-byte
// strides, so every word is aligned.  The heads of several records can be
// read at once; r <= 0 reads the zero guard record.
struct RecHead {
    unsigned long long w[4];
};
__device__ __forceinline__ RecHead rec_head(const Dev &D, int r)
{
    const unsigned long long *p = reinterpret_cast<const unsigned long long *>(D.rec + (r > 0 ? r : 0));
    return RecHead{{p[0], p[1], p[2], p[3]}};
}
// the k-th int16 of the head (little-endian: bytes 2k, 2k + 1)
__device__ __forceinline__ int head16(const RecHead &h, int k)
{
    return (int)(int16_t)(unsigned short)(h.w[k >> 2] >> (16 * (k & 3)));
}
// whether the head's NextN list (int16 3..14) holds s
__device__ __forceinline__ bool head_lists(const RecHead &h, P3 s)
{
    bool hit = false;
#pragma unroll
    for (int i = 0; i < 4; i++)
        hit |= head16(h, 3 + 3 * i) == s.x && head16(h, 4 + 3 * i) == s.y && head16(h, 5 + 3 * i) == s.z;
    return hit;
}
__device__ __forceinline__ bool rec_lists(const Dev &D, int r, P3 s) { return head_lists(rec_head(D, r), s); }

// the selection weight of a record in its tile list
__device__ __forceinline__ float list_rate(const Rec &R)
{
    return R.ev == EV_NONE ? 0.f : (R.ev == EV_ISO ? -1.f : R.rate);
}


// Get_Prob (Get_Prob.f:54-331) without coverage: the event code and FP32 rate
// of a site from its LattCoo word and NextN.  An empty site carries the sum
// of the deposition rates (the species is drawn when the event happens, from
// the same shares as Get_Prob.f:159-176 draws it); an isolated atom gets code
// EV_ISO, its rate 1e5 x the total being set at selection (:300-306).
__device__ void get_prob(const Dev &D, int occ, int nsic, int coor, P3 site, const P3 nn[4], uint8_t &ev, float &rate)
{
    if (!occ) {
        if (coor == 1) {
            int cnn = coor_of(cw(D, nn[0]));
            if (cnn >= 2) {
                ev = EV_DEP;
                rate = D.pds[0];
            } else {
                ev = EV_DUMMY;        // Get_Prob.f:181-184
                rate = 1.e-8f;
            }
        } else if (coor == 2 || coor == 3) {
            ev = EV_DEP;
            rate = D.pds[coor - 1];
        } else {
            ev = EV_NONE;
            rate = 0.f;
        }
        return;
    }
    // the four NextN words and records are read first, all in flight at once,
    // then tested: a chain of two memory round trips instead of three per
    // neighbour one after the other
    uint32_t v[4];
    int rn[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
        const int64_t g = gidx(D, nn[i]);
        v[i] = D.coo[g];
        rn[i] = D.ind[g];
    }
    RecHead h[4];
#pragma unroll
    for (int i = 0; i < 4; i++) h[i] = rec_head(D, rn[i]);
    bool bond[4];
#pragma unroll
    for (int i = 0; i < 4; i++)                              // reciprocal bonds only (:232-239)
        bond[i] = occ_of(v[i]) && cov_of(v[i]) != WALLIND && head_lists(h[i], site);
    int nsi = 0, nc = 0, nb = 0, nw = 0;
#pragma unroll
    for (int i = 0; i < 4; i++) {
        if (!occ_of(v[i])) continue;
        if (cov_of(v[i]) == WALLIND) {
            nw++;
            continue;
        }
        if (bond[i]) {
            int s = sp_of(v[i]);
            nsi += s == 1;
            nc += s == 2;
            nb += s == 3;
        }
    }
    int tot = nsi + nc + nb + nw;
    if (tot != coor) {                                      // :293-298
        set_err(D, E_INVARIANT, site.x, site.y, site.z);
        ev = EV_NONE;
        rate = 0.f;
        return;
    }
    if (tot > 3) {
        ev = EV_NONE;
        rate = 0.f;
    } else if (tot == 0) {
        ev = EV_ISO;
        rate = 0.f;
    } else {
        int s = nsic >= 1 && nsic <= 3 ? nsic : 1;
        ev = EV_EVAP;
        rate = D.pef[(s - 1) * 64 + (nsi + nw) * 16 + nc * 4 + nb];
    }
}

// ---- list bookkeeping (AddMC / EraseMC and friends, Add.f, Erase.f) ----
// A site that gets an event joins its tile's list in an order that does not
// depend on the scheduling of warps or lanes, so a run is reproducible for
// its seed: a site of the running tile is appended after the event, in lane
// order (flush_pending); a site of an idle neighbour tile goes to that tile's
// inbox, which the tile drains at its next phase in grid-point order.
__device__ void list_site(const Dev &D, Ctx &c, int r)
{
    if (c.tile < 0) return;               // replay: the lists are rebuilt before a run
    Rec &R = D.rec[r];
    if (R.flags & F_LISTED) return;
    int t = tile_of(D, R.x, R.y);
    if (t == c.tile) {
        if (c.npend >= 4) {
            set_err(D, E_INVARIANT, R.x, R.y, R.z);
            return;
        }
        c.pend[c.npend++] = r;
        R.flags |= F_LISTED | F_PEND;
        return;
    }
    int k = atomicAdd(&D.ib_n[t], 1);
    if (k >= ICAP) {
        set_err(D, E_CAPACITY, t, k, 2);
        return;
    }
    D.ib[(int64_t)t * ICAP + k] = r;
    R.flags |= F_LISTED | F_INBOX;
}

__device__ void set_event(const Dev &D, Ctx &c, int r, uint8_t ev, float rate)
{
    if (r <= 0) {
        set_err(D, E_INVARIANT, -1, r, 0);
        return;
    }
    Rec &R = D.rec[r];
    c.dmc += (ev != 0) - (R.ev != 0);
    R.ev = ev;
    R.rate = rate;
    if (c.tile < 0) return;               // replay: the lists are rebuilt before a run
    if (R.flags & F_LISTED) {
        if (!(R.flags & (F_PEND | F_INBOX))) D.tr[(int64_t)tile_of(D, R.x, R.y) * LCAP + R.slot] = list_rate(R);
    } else if (ev) {
        list_site(D, c, r);
    }
}

// A record from the running tile's reusable stack, else a new one.  The
// lanes of a warp may allocate at once (the neighbour updates of one event
// run on four lanes): the stack is popped atomically, and nothing pushes to
// it during a phase.
__device__ int alloc_rec(const Dev &D, const Ctx &c)
{
    int t = c.tile < 0 ? 0 : c.tile;
    int n = atomicSub(&D.fr_n[t], 1);
    if (n > 0) return D.fr[(int64_t)t * FCAP + n - 1];
    atomicAdd(&D.fr_n[t], 1);
    int r = atomicAdd(D.top, 1);
    if (r >= D.rcap) {
        set_err(D, E_CAPACITY, -2, r, 0);
        return 0;
    }
    return r;
}

__device__ void free_rec(const Dev &D, const Ctx &c, int r)
{
    if (c.tile < 0) {                     // replay: reusable at once (no lists)
        int n = D.fr_n[0];
        if (n < FCAP) {
            D.fr[n] = r;
            D.fr_n[0] = n + 1;
        }
        return;
    }
    int n = atomicAdd(&D.fp_n[c.tile], 1);   // a full stack drops the record (counted past FCAP)
    if (n < FCAP) D.fp[(int64_t)c.tile * FCAP + n] = r;
}

// a new listed site (AddMC of a coor-1 empty site, Add.f:24-52)
__device__ void new_site(const Dev &D, Ctx &c, P3 p, const P3 nn[4], uint8_t ev, float rate)
{
    int r = alloc_rec(D, c);
    if (r <= 0) return;
    Rec &R = D.rec[r];
    R.x = (int16_t)p.x;
    R.y = (int16_t)p.y;
    R.z = (int16_t)p.z;
    for (int i = 0; i < 4; i++) put_nn(R, i, nn[i]);
    R.ev = EV_NONE;
    R.flags = 0;
    R.rate = 0.f;
    D.ind[gidx(D, p)] = r;
    set_event(D, c, r, ev, rate);
}

// the site leaves every list (EraseMC with LattInd = 0, Erase.f:24-76)
__device__ void drop_site(const Dev &D, Ctx &c, P3 p)
{
    int64_t g = gidx(D, p);
    int r = D.ind[g];
    if (r <= 0) {
        set_err(D, E_INVARIANT, p.x, p.y, p.z);
        return;
    }
    D.ind[g] = 0;
    Rec &R = D.rec[r];
    c.dmc -= R.ev != 0;
    if (c.tile >= 0 && (R.flags & F_LISTED) && !(R.flags & (F_PEND | F_INBOX)))
        D.tr[(int64_t)tile_of(D, R.x, R.y) * LCAP + R.slot] = 0.f;
    R.ev = EV_NONE;
    R.flags = 0;
    R.rate = 0.f;
    R.x = -1;
    free_rec(D, c, r);
}

// ---- geometry: FIND_SN.f:26-84, FIND_NN.f:25-77, IF_Arm_Choice.f:21-56 ----
// FP64 as the reference, each product and sum rounded on its own (no fused
// multiply-add), NINT to the grid.
// NINT of v when the FP32 value v32 (within 1e-3 of v) is not near a
// rounding half: the two round alike; -2^30 otherwise (take the FP64 form)
__device__ __forceinline__ int nint_safe(float v32)
{
    const float f = fabsf(v32 - truncf(v32));
    return fabsf(f - 0.5f) < 1.0e-3f ? -(1 << 30) : (int)rintf(v32);
}

__device__ void find_sn_fp64(const Dev &D, P3 site, P3 sitec, const P3 sn_in[3], P3 zig[3], P3 arm[3]);

// FIND_SN in FP32 where that gives the FP64 result: the zig-zag sites are
// integer arithmetic (2 cent - sn = site + sitec - sn); an arm-chair
// coordinate sn + shift ax rounds as in FP64 unless the FP32 value lies
// within 1e-3 of a half (FP32's error here is below 1e-4), and then the FP64
// form runs.  GB300's FP64 rate is a small fraction of its FP32 rate.
__device__ void find_sn(const Dev &D, P3 site, P3 sitec, const P3 sn_in[3], P3 zig[3], P3 arm[3])
{
    const int lx = D.lx, ly = D.ly;
    P3 sn[3] = {sn_in[0], sn_in[1], sn_in[2]};
    P3 c = sitec;
    if (abs(site.x - c.x) > lx / 2) c.x += isign(lx, site.x - c.x);
    if (abs(site.y - c.y) > ly / 2) c.y += isign(ly, site.y - c.y);
    for (int i = 0; i < 3; i++) {
        if (abs(site.x - sn[i].x) > lx / 2) sn[i].x += isign(lx, site.x - sn[i].x);
        if (abs(site.y - sn[i].y) > ly / 2) sn[i].y += isign(ly, site.y - sn[i].y);
    }
    const int d3[3] = {site.x - c.x, site.y - c.y, site.z - c.z};
    const float inv = 1.0f / sqrtf((float)(d3[0] * d3[0] + d3[1] * d3[1] + d3[2] * d3[2]));
    const float sh = (float)D.shift;
    int off[3];
    for (int k = 0; k < 3; k++) {
        off[k] = nint_safe(sh * ((float)d3[k] * inv));
        if (off[k] == -(1 << 30)) {
            find_sn_fp64(D, site, sitec, sn_in, zig, arm);
            return;
        }
    }
    for (int i = 0; i < 3; i++) {
        zig[i] = P3{site.x + c.x - sn[i].x, site.y + c.y - sn[i].y, site.z + c.z - sn[i].z};
        arm[i] = P3{sn[i].x + off[0], sn[i].y + off[1], sn[i].z + off[2]};
        if (zig[i].x >= lx) zig[i].x -= lx;
        if (zig[i].x < 0) zig[i].x += lx;
        if (zig[i].y >= ly) zig[i].y -= ly;
        if (zig[i].y < 0) zig[i].y += ly;
        if (arm[i].x >= lx) arm[i].x -= lx;
        if (arm[i].x < 0) arm[i].x += lx;
        if (arm[i].y >= ly) arm[i].y -= ly;
        if (arm[i].y < 0) arm[i].y += ly;
    }
}

__device__ void find_sn_fp64(const Dev &D, P3 site, P3 sitec, const P3 sn_in[3], P3 zig[3], P3 arm[3])
{
    const int lx = D.lx, ly = D.ly;
    P3 sn[3] = {sn_in[0], sn_in[1], sn_in[2]};
    if (abs(site.x - sitec.x) > lx / 2) sitec.x += isign(lx, site.x - sitec.x);
    if (abs(site.y - sitec.y) > ly / 2) sitec.y += isign(ly, site.y - sitec.y);
    for (int i = 0; i < 3; i++) {
        if (abs(site.x - sn[i].x) > lx / 2) sn[i].x += isign(lx, site.x - sn[i].x);
        if (abs(site.y - sn[i].y) > ly / 2) sn[i].y += isign(ly, site.y - sn[i].y);
    }
    const int s3[3] = {site.x, site.y, site.z}, c3[3] = {sitec.x, sitec.y, sitec.z};
    double cent[3], ax[3];
    for (int k = 0; k < 3; k++) {
        cent[k] = 0.5 * ((double)c3[k] + (double)s3[k]);     // exact
        ax[k] = (double)s3[k] - (double)c3[k];
    }
    double snorm = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);   // integer squares: exact sum
    for (int k = 0; k < 3; k++) ax[k] = __ddiv_rn(ax[k], snorm);
    for (int i = 0; i < 3; i++) {
        const int n3[3] = {sn[i].x, sn[i].y, sn[i].z};
        int z3[3], a3[3];
        for (int k = 0; k < 3; k++) {
            z3[k] = nint(2.0 * cent[k] - (double)n3[k]);          // exact
            a3[k] = nint(__dadd_rn((double)n3[k], __dmul_rn(D.shift, ax[k])));
        }
        zig[i] = P3{z3[0], z3[1], z3[2]};
        arm[i] = P3{a3[0], a3[1], a3[2]};
        if (zig[i].x >= lx) zig[i].x -= lx;
        if (zig[i].x < 0) zig[i].x += lx;
        if (zig[i].y >= ly) zig[i].y -= ly;
        if (zig[i].y < 0) zig[i].y += ly;
        if (arm[i].x >= lx) arm[i].x -= lx;
        if (arm[i].x < 0) arm[i].x += lx;
        if (arm[i].y >= ly) arm[i].y -= ly;
        if (arm[i].y < 0) arm[i].y += ly;
    }
}

__device__ void find_nn_fp64(const Dev &D, P3 s1, P3 s2, P3 sc, P3 out[2]);

// FIND_NN in FP32 where that gives the FP64 result (see find_sn); the
// rotated coordinates are at most a bond long, FP32's error below 1e-5
__device__ void find_nn(const Dev &D, P3 s1, P3 s2, P3 sc, P3 out[2])
{
    const int lx = D.lx, ly = D.ly;
    P3 a = s1, b = s2;
    if (abs(sc.x - a.x) > lx / 2) a.x += isign(lx, sc.x - a.x);
    if (abs(sc.y - a.y) > ly / 2) a.y += isign(ly, sc.y - a.y);
    if (abs(sc.x - b.x) > lx / 2) b.x += isign(lx, sc.x - b.x);
    if (abs(sc.y - b.y) > ly / 2) b.y += isign(ly, sc.y - b.y);
    const int d3[3] = {sc.x - a.x, sc.y - a.y, sc.z - a.z};
    const float t3[3] = {(float)(b.x - sc.x), (float)(b.y - sc.y), (float)(b.z - sc.z)};
    const float inv = 1.0f / sqrtf((float)(d3[0] * d3[0] + d3[1] * d3[1] + d3[2] * d3[2]));
    const float ax[3] = {(float)d3[0] * inv, (float)d3[1] * inv, (float)d3[2] * inv};
    const int c3[3] = {sc.x, sc.y, sc.z};
    for (int irot = 0; irot < 2; irot++) {
        const float cth = (float)D.cth[irot], sth = (float)D.sth[irot], omc = 1.0f - cth;
        float rot[3][3];
        for (int i = 0; i < 3; i++) rot[i][i] = ax[i] * ax[i] * omc + cth;
        rot[1][0] = ax[0] * ax[1] * omc - ax[2] * sth;
        rot[0][1] = ax[0] * ax[1] * omc + ax[2] * sth;
        rot[2][0] = ax[0] * ax[2] * omc + ax[1] * sth;
        rot[0][2] = ax[0] * ax[2] * omc - ax[1] * sth;
        rot[2][1] = ax[1] * ax[2] * omc - ax[0] * sth;
        rot[1][2] = ax[1] * ax[2] * omc + ax[0] * sth;
        int o3[3];
        for (int k = 0; k < 3; k++) {
            const int q = nint_safe(rot[0][k] * t3[0] + rot[1][k] * t3[1] + rot[2][k] * t3[2]);
            if (q == -(1 << 30)) {
                find_nn_fp64(D, s1, s2, sc, out);
                return;
            }
            o3[k] = q + c3[k];
        }
        P3 p{o3[0], o3[1], o3[2]};
        if (p.x >= lx) p.x -= lx;
        if (p.x < 0) p.x += lx;
        if (p.y >= ly) p.y -= ly;
        if (p.y < 0) p.y += ly;
        out[irot] = p;
    }
}

__device__ void find_nn_fp64(const Dev &D, P3 s1, P3 s2, P3 sc, P3 out[2])
{
    const int lx = D.lx, ly = D.ly;
    if (abs(sc.x - s1.x) > lx / 2) s1.x += isign(lx, sc.x - s1.x);
    if (abs(sc.y - s1.y) > ly / 2) s1.y += isign(ly, sc.y - s1.y);
    if (abs(sc.x - s2.x) > lx / 2) s2.x += isign(lx, sc.x - s2.x);
    if (abs(sc.y - s2.y) > ly / 2) s2.y += isign(ly, sc.y - s2.y);
    const int c3[3] = {sc.x, sc.y, sc.z}, t3[3] = {s2.x, s2.y, s2.z};
    double ax[3] = {(double)(sc.x - s1.x), (double)(sc.y - s1.y), (double)(sc.z - s1.z)};
    double snorm = sqrt(ax[0] * ax[0] + ax[1] * ax[1] + ax[2] * ax[2]);
    for (int k = 0; k < 3; k++) ax[k] = __ddiv_rn(ax[k], snorm);
    for (int irot = 0; irot < 2; irot++) {
        const double cth = D.cth[irot], sth = D.sth[irot];
        const double omc = __dsub_rn(1.0, cth);
        double rot[3][3];
        for (int i = 0; i < 3; i++) rot[i][i] = __dadd_rn(__dmul_rn(__dmul_rn(ax[i], ax[i]), omc), cth);
        rot[1][0] = __dsub_rn(__dmul_rn(__dmul_rn(ax[0], ax[1]), omc), __dmul_rn(ax[2], sth));
        rot[0][1] = __dadd_rn(__dmul_rn(__dmul_rn(ax[0], ax[1]), omc), __dmul_rn(ax[2], sth));
        rot[2][0] = __dadd_rn(__dmul_rn(__dmul_rn(ax[0], ax[2]), omc), __dmul_rn(ax[1], sth));
        rot[0][2] = __dsub_rn(__dmul_rn(__dmul_rn(ax[0], ax[2]), omc), __dmul_rn(ax[1], sth));
        rot[2][1] = __dsub_rn(__dmul_rn(__dmul_rn(ax[1], ax[2]), omc), __dmul_rn(ax[0], sth));
        rot[1][2] = __dadd_rn(__dmul_rn(__dmul_rn(ax[1], ax[2]), omc), __dmul_rn(ax[0], sth));
        int o3[3];
        for (int k = 0; k < 3; k++) {
            double r = 0.0;
            for (int l = 0; l < 3; l++) r = __dadd_rn(r, __dmul_rn(rot[l][k], (double)(t3[l] - c3[l])));
            o3[k] = nint(r) + c3[k];
        }
        P3 p{o3[0], o3[1], o3[2]};
        if (p.x >= lx) p.x -= lx;
        if (p.x < 0) p.x += lx;
        if (p.y >= ly) p.y -= ly;
        if (p.y < 0) p.y += ly;
        out[irot] = p;
    }
}

__device__ float tie_uniform(const Dev &D, Ctx &c)
{
    U4 r = philox4x32_10(U4{c.nties++, (uint32_t)c.tile, c.key2, c.key3}, D.k0 ^ 0x5bd1e995u, D.k1);
    return u01(r.x);
}

// 1 for arm-chair (hexagonal), 0 for zig-zag (cubic)
__device__ int arm_choice(const Dev &D, Ctx &c, const P3 zig[3], const P3 arm[3])
{
    int ca = 0, cz = 0;
    for (int i = 0; i < 3; i++) {
        ca += coor_of(cw(D, arm[i]));
        cz += coor_of(cw(D, zig[i]));
    }
    int choice;
    if (cz > ca) choice = 0;
    else if (cz == ca) {
        if (c.tile < 0) return c.forced_arm;
        choice = (double)tie_uniform(D, c) <= D.pzig ? 0 : 1;
    } else choice = 1;
    if (c.tile < 0 && choice != c.forced_arm) set_err(D, E_ARM, ca, cz, c.forced_arm);
    return choice;
}

// ---- events ----
// Neighbour i (NextN entry n) of a deposition at `site`, deposition.f:
// 78-235.  Returns the change of the site's own coordination that this
// neighbour makes: a wall, or an atom that lists the site when the site had
// coordination 1 (then only for i >= 1).  It reads and writes n, n's record
// and n's own neighbours' words only: two neighbours of a site are never
// bonded, so the four calls of one event are independent of one another.
__device__ int dep_neighbour(const Dev &D, Ctx &c, P3 site, int coor_old, int i, P3 n)
{
    int inc = 0;
    const int64_t gn = gidx(D, n);
    const uint32_t vn = D.coo[gn];
    const int rn = D.ind[gn];
    int coornn = coor_of(vn);
    const int covind = cov_of(vn);
    uint8_t ev;
    float rate;
    if (!occ_of(vn)) {
        if (coornn == 0) {                             // :86-99
            D.coo[gn] = with_coor(vn, 1);
            P3 nnn[4] = {site, {0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
            get_prob(D, 0, 0, 1, n, nnn, ev, rate);
            if (ev) new_site(D, c, n, nnn, ev, rate);
        } else if (coornn == 1) {                      // :100-160
            if (rn <= 0) {
                set_err(D, E_INVARIANT, n.x, n.y, n.z);
                return 0;
            }
            Rec &N = D.rec[rn];
            P3 nnn[4];
            load_nn(N, nnn);
            int dx = abs(nnn[0].x - site.x);
            if (D.lx - dx < dx) dx = D.lx - dx;
            int dy = abs(nnn[0].y - site.y);
            if (D.ly - dy < dy) dy = D.ly - dy;
            int dz = nnn[0].z - site.z;
            if (dx * dx + dy * dy + dz * dz == 72) {
                coornn = 2;
                nnn[1] = site;
                P3 ns[2];
                find_nn(D, nnn[0], nnn[1], n, ns);
                // both candidates' words and records in flight at once
                uint32_t v[2];
                int rk[2];
#pragma unroll
                for (int k = 0; k < 2; k++) {
                    nnn[k + 2] = ns[k];
                    const int64_t g = gidx(D, ns[k]);
                    v[k] = D.coo[g];
                    rk[k] = D.ind[g];
                }
                const RecHead h0 = rec_head(D, rk[0]), h1 = rec_head(D, rk[1]);
                if (occ_of(v[0]) && coor_of(v[0]) <= 3 && cov_of(v[0]) != WALLIND && head_lists(h0, n)) coornn++;
                if (occ_of(v[1]) && coor_of(v[1]) <= 3 && cov_of(v[1]) != WALLIND && head_lists(h1, n)) coornn++;
                D.coo[gn] = with_coor(vn, coornn);
                for (int k = 0; k < 4; k++) put_nn(N, k, nnn[k]);
                get_prob(D, 0, 0, coornn, n, nnn, ev, rate);
                set_event(D, c, rn, ev, rate);         // no event: EraseMC + AddVoid
            }
        } else if (coornn == 2 || coornn == 3) {       // :161-191
            if (rn <= 0) {
                set_err(D, E_INVARIANT, n.x, n.y, n.z);
                return 0;
            }
            P3 nnn[4];
            load_nn(D.rec[rn], nnn);
            if (in_list(nnn, site)) {
                coornn++;
                D.coo[gn] = with_coor(vn, coornn);
                get_prob(D, 0, 0, coornn, n, nnn, ev, rate);
                set_event(D, c, rn, ev, rate);
            }
        }
    } else if (covind != WALLIND) {                    // :192-230
        if (covind != 0) {
            set_err(D, E_INVARIANT, n.x, n.y, n.z);
            return 0;
        }
        if (coornn <= 3) {
            if (rn <= 0) {
                set_err(D, E_INVARIANT, n.x, n.y, n.z);
                return 0;
            }
            P3 nnn[4];
            load_nn(D.rec[rn], nnn);
            if (in_list(nnn, site)) {
                coornn++;
                D.coo[gn] = with_coor(vn, coornn);
                get_prob(D, 1, sp_of(vn), coornn, n, nnn, ev, rate);
                set_event(D, c, rn, ev, rate);         // no event: EraseMC + AddBulk
                if (coor_old == 1 && i >= 1) inc = 1;
            }
        }
    } else {
        inc = 1;                                       // a wall
    }
    return inc;
}

// Deposition of species sp on the empty site (deposition.f:24-251)
__device__ void deposition(const Dev &D, Ctx &c, P3 site, int sp)
{
    const int64_t gs = gidx(D, site);
    const int rs = D.ind[gs];
    if (rs <= 0) {
        set_err(D, E_INVARIANT, site.x, site.y, site.z);
        return;
    }
    uint32_t w = D.coo[gs];
    int coor = coor_of(w);
    const int coor_old = coor;
    w = (w & ~(7u << 27)) | B_OCC | ((uint32_t)sp << 27);
    D.coo[gs] = w;
    Rec &R = D.rec[rs];
    if (coor == 1) {                                       // :49-74
        P3 sitec = nn_at(R, 0);
        const Rec &Rc = D.rec[D.ind[gidx(D, sitec)]];
        P3 sn[3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
        int j = 0;
        for (int i = 0; i < 4; i++) {
            P3 q = nn_at(Rc, i);
            if (!same(q, site)) {
                if (j < 3) sn[j] = q;
                j++;
            }
        }
        P3 zig[3], arm[3];
        find_sn(D, site, sitec, sn, zig, arm);
        int a = arm_choice(D, c, zig, arm);
        for (int i = 0; i < 3; i++) put_nn(R, i + 1, a ? arm[i] : zig[i]);
    }
    P3 nextn[4];
    load_nn(R, nextn);
    for (int i = 0; i < 4; i++) {                          // :78-235
        coor += dep_neighbour(D, c, site, coor_old, i, nextn[i]);
        if (*(volatile int32_t *)D.err) return;
    }
    if (coor != coor_old) D.coo[gs] = with_coor(D.coo[gs], coor);   // :236-250
    uint8_t ev;
    float rate;
    get_prob(D, 1, sp, coor, site, nextn, ev, rate);
    set_event(D, c, D.ind[gs], ev, rate);
}

// The neighbour of `site` whose list holds `site`, among the occupied
// non-wall sites of nn (Evaporation.f:87-104,238-253); NBuff keeps the last.
__device__ void prune_to_buffer(const Dev &D, Ctx &c, Rec &S, P3 site, bool &got)
{
    // the neighbours' words and records are read before S changes (none of
    // them is S: a site is not its own neighbour), all in flight at once
    P3 q[4];
    uint32_t v[4];
    int rq[4];
#pragma unroll
    for (int j = 0; j < 4; j++) {
        q[j] = nn_at(S, j);
        const int64_t g = gidx(D, q[j]);
        v[j] = D.coo[g];
        rq[j] = D.ind[g];
    }
    RecHead h[4];
#pragma unroll
    for (int j = 0; j < 4; j++) h[j] = rec_head(D, rq[j]);
    bool hit[4];
#pragma unroll
    for (int j = 0; j < 4; j++)
        hit[j] = occ_of(v[j]) && coor_of(v[j]) <= 3 && cov_of(v[j]) != WALLIND && head_lists(h[j], site);
    for (int j = 0; j < 4; j++) {
        if (hit[j]) {
            c.nbuff = q[j];
            got = true;
        }
        put_nn(S, j, P3{0, 0, 0});
    }
    put_nn(S, 0, c.nbuff);
}

// NextN entry n of an evaporating atom at `site`, Evaporation.f:46-215.
// Returns -1 for a wall (the site's coordination drops), else 0.  Touches n,
// n's record and reads n's neighbours only (independent of the other three,
// as in deposition); the NBuff of a pruned coor-1 site is this call's (the
// run treats a stale NBuff as an error, the replay carries it as the
// reference does).
__device__ int evap_neighbour(const Dev &D, Ctx &c, P3 site, P3 n)
{
    const int64_t gn = gidx(D, n);
    const uint32_t vn = D.coo[gn];
    const int rn = D.ind[gn];
    int coornn = coor_of(vn);
    const int covind = cov_of(vn);
    uint8_t ev;
    float rate;
    if (!occ_of(vn)) {
        if (coornn < 1 || coornn > 4) return 0;
        if (rn <= 0) {                                 // a coordinated empty site is always listed
            set_err(D, E_INVARIANT, n.x, n.y, n.z);
            return 0;
        }
        P3 nnn[4];
        load_nn(D.rec[rn], nnn);
        if (!in_list(nnn, site)) return 0;
        if (coornn == 1) {                             // :51-68
            drop_site(D, c, n);
            D.coo[gn] = 0;
        } else if (coornn == 2) {                      // :69-123
            D.coo[gn] = with_coor(vn, 1);
            bool got = false;
            prune_to_buffer(D, c, D.rec[rn], n, got);
            if (!got && c.tile >= 0) set_err(D, E_NBUFF, n.x, n.y, n.z);
            get_prob(D, 0, 0, 1, n, nnn, ev, rate);   // the list as it was before pruning
            set_event(D, c, rn, ev, rate);
        } else {                                       // :124-164 (coor 3 -> 2, void -> MC)
            coornn--;
            D.coo[gn] = with_coor(vn, coornn);
            get_prob(D, 0, 0, coornn, n, nnn, ev, rate);
            set_event(D, c, rn, ev, rate);
        }
    } else if (covind != WALLIND) {                    // :166-210
        if (covind != 0 || rn <= 0) {
            set_err(D, E_INVARIANT, n.x, n.y, n.z);
            return 0;
        }
        P3 nnn[4];
        load_nn(D.rec[rn], nnn);
        if (in_list(nnn, site)) {
            coornn--;
            D.coo[gn] = with_coor(vn, coornn);
            get_prob(D, 1, sp_of(vn), coornn, n, nnn, ev, rate);
            set_event(D, c, rn, ev, rate);             // bulk -> MC when coor was 4
        }
    } else {
        return -1;                                     // a wall
    }
    return 0;
}

// Evaporation of the atom at site (Evaporation.f:25-262)
__device__ void evaporation(const Dev &D, Ctx &c, P3 site)
{
    const int64_t gs = gidx(D, site);
    const int rs = D.ind[gs];
    if (rs <= 0) {
        set_err(D, E_INVARIANT, site.x, site.y, site.z);
        return;
    }
    uint32_t w = D.coo[gs];
    int coor = coor_of(w);
    D.coo[gs] = w & ~(B_OCC | (7u << 27));
    P3 nextn[4];
    load_nn(D.rec[rs], nextn);
    for (int i = 0; i < 4; i++) {
        coor += evap_neighbour(D, c, site, nextn[i]);
        if (*(volatile int32_t *)D.err) return;
    }
    D.coo[gs] = with_coor(D.coo[gs], coor);                // :216-261
    if (coor == 0) {
        drop_site(D, c, site);
        return;
    }
    uint8_t ev;
    float rate;
    get_prob(D, 0, 0, coor, site, nextn, ev, rate);
    Rec &S = D.rec[D.ind[gs]];
    if (coor == 1) {
        bool got = false;
        prune_to_buffer(D, c, S, site, got);
        if (!got && c.tile >= 0) set_err(D, E_NBUFF, site.x, site.y, site.z);
    }
    set_event(D, c, D.ind[gs], ev, rate);
}

// ---- kernels ----
constexpr unsigned FULL = 0xffffffffu;

// The same events with the four neighbour updates on lanes 1..4 at once
// (all lanes of the warp call these).  Lane 0 updates the event site first
// (deposition.f:43-74: occupancy, species and the stacking of a coor-1
// site) and last (:236-250, Evaporation.f:216-261), the lanes between: their
// updates touch disjoint words (two NextN sites of a site are never bonded),
// and their changes of the site's coordination are summed.  A site whose
// NextN list repeats a grid point (left by the reference's rounding only in
// contrived geometry) takes the serial order.
__device__ bool nn_distinct(const P3 nn[4])
{
    for (int i = 0; i < 4; i++)
        for (int j = i + 1; j < 4; j++)
            if (same(nn[i], nn[j])) return false;
    return true;
}

__device__ void deposition_warp(const Dev &D, Ctx &c, P3 site, int sp, int lane)
{
    const int64_t gs = gidx(D, site);
    int coor_old = 0, go = 0;
    if (lane == 0) {
        const int rs = D.ind[gs];
        if (rs <= 0) {
            set_err(D, E_INVARIANT, site.x, site.y, site.z);
        } else {
            uint32_t w = D.coo[gs];
            coor_old = coor_of(w);
            D.coo[gs] = (w & ~(7u << 27)) | B_OCC | ((uint32_t)sp << 27);
            Rec &R = D.rec[rs];
            if (coor_old == 1) {                           // :49-74
                P3 sitec = nn_at(R, 0);
                const Rec &Rc = D.rec[D.ind[gidx(D, sitec)]];
                P3 sn[3] = {{0, 0, 0}, {0, 0, 0}, {0, 0, 0}};
                int j = 0;
                for (int i = 0; i < 4; i++) {
                    P3 q = nn_at(Rc, i);
                    if (!same(q, site)) {
                        if (j < 3) sn[j] = q;
                        j++;
                    }
                }
                P3 zig[3], arm[3];
                find_sn(D, site, sitec, sn, zig, arm);
                int a = arm_choice(D, c, zig, arm);
                for (int i = 0; i < 3; i++) put_nn(R, i + 1, a ? arm[i] : zig[i]);
            }
            P3 nn[4];
            load_nn(R, nn);
            go = nn_distinct(nn) ? 1 : 2;
        }
    }
    go = __shfl_sync(FULL, go, 0);
    coor_old = __shfl_sync(FULL, coor_old, 0);
    __syncwarp();
    if (!go) return;
    P3 nextn[4];
    load_nn(D.rec[D.ind[gs]], nextn);
    int inc = 0;
    if (go == 1) {
        if (lane >= 1 && lane <= 4) inc = dep_neighbour(D, c, site, coor_old, lane - 1, nextn[lane - 1]);
    } else if (lane == 0) {
        for (int i = 0; i < 4; i++) inc += dep_neighbour(D, c, site, coor_old, i, nextn[i]);
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) inc += __shfl_xor_sync(FULL, inc, o);   // lanes 0..7 hold the sum
    __syncwarp();
    if (lane == 0 && !block_err()) {
        const int coor = coor_old + inc;
        if (coor != coor_old) D.coo[gs] = with_coor(D.coo[gs], coor);    // :236-250
        uint8_t ev;
        float rate;
        get_prob(D, 1, sp, coor, site, nextn, ev, rate);
        set_event(D, c, D.ind[gs], ev, rate);
    }
    __syncwarp();
}

__device__ void evaporation_warp(const Dev &D, Ctx &c, P3 site, int lane)
{
    const int64_t gs = gidx(D, site);
    int coor_old = 0, go = 0;
    if (lane == 0) {
        const int rs = D.ind[gs];
        if (rs <= 0) {
            set_err(D, E_INVARIANT, site.x, site.y, site.z);
        } else {
            uint32_t w = D.coo[gs];
            coor_old = coor_of(w);
            D.coo[gs] = w & ~(B_OCC | (7u << 27));
            P3 nn[4];
            load_nn(D.rec[rs], nn);
            go = nn_distinct(nn) ? 1 : 2;
        }
    }
    go = __shfl_sync(FULL, go, 0);
    coor_old = __shfl_sync(FULL, coor_old, 0);
    __syncwarp();
    if (!go) return;
    P3 nextn[4];
    load_nn(D.rec[D.ind[gs]], nextn);
    int dec = 0;
    if (go == 1) {
        if (lane >= 1 && lane <= 4) dec = evap_neighbour(D, c, site, nextn[lane - 1]);
    } else if (lane == 0) {
        for (int i = 0; i < 4; i++) dec += evap_neighbour(D, c, site, nextn[i]);
    }
#pragma unroll
    for (int o = 4; o > 0; o >>= 1) dec += __shfl_xor_sync(FULL, dec, o);
    __syncwarp();
    if (lane == 0 && !block_err()) {
        const int coor = coor_old + dec;
        D.coo[gs] = with_coor(D.coo[gs], coor);                          // :216-261
        if (coor == 0) {
            drop_site(D, c, site);
        } else {
            uint8_t ev;
            float rate;
            get_prob(D, 0, 0, coor, site, nextn, ev, rate);
            Rec &S = D.rec[D.ind[gs]];
            if (coor == 1) {
                bool got = false;
                prune_to_buffer(D, c, S, site, got);
                if (!got) set_err(D, E_NBUFF, site.x, site.y, site.z);
            }
            set_event(D, c, D.ind[gs], ev, rate);
        }
    }
    __syncwarp();
}

// Apply event code ev of record r: the deposited species is drawn from the
// PTransD shares of the site's coordination with u (Get_Prob.f:159-176);
// an unsupported coor-1 site deposits species 1 (:181-184).
__device__ void apply_warp(const Dev &D, Ctx &c, int r, float u, int lane)
{
    const Rec &R = D.rec[r];
    const P3 site{R.x, R.y, R.z};
    const uint8_t ev = R.ev;
    __syncwarp();
    if (ev == EV_EVAP || ev == EV_ISO) {
        evaporation_warp(D, c, site, lane);
        return;
    }
    int sp = 1;
    if (ev == EV_DEP) {
        int co = coor_of(cw(D, site));
        co = co < 1 ? 1 : (co > 3 ? 3 : co);
        sp = u < D.pds[3 + 2 * (co - 1)] ? 1 : (u < D.pds[4 + 2 * (co - 1)] ? 2 : 3);
    }
    deposition_warp(D, c, site, sp, lane);
}

__device__ __forceinline__ unsigned lanemask_lt() { return (1u << (threadIdx.x & 31)) - 1u; }

// One colour phase: every tile of the colour runs from the window's start to
// its end (one warp per tile).
__device__ __forceinline__ long long site_key(const Dev &D, const Rec &R)
{
    return ((long long)(R.z + ZG) * D.ly + R.y) * D.lx + R.x;
}

// The running tile's sites that got an event in this event, appended in
// lane order (every lane calls this after the event).  A record dropped or
// left without an event in the meantime is appended as a dead entry (rate 0)
// for the next compaction.  ntl is the list's length, held by the warp: only
// the tile's own warp appends to its list during a phase (other tiles' warps
// write its inbox), so the length needs no atomic; lane 0 stores it back.
__device__ void flush_pending(const Dev &D, Ctx &c, int t, int lane, int &ntl)
{
    int inc = c.npend;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(FULL, inc, o);
        if (lane >= o) inc += y;
    }
    const int tot = __shfl_sync(FULL, inc, 31);
    if (!tot) return;
    const int base = ntl;
    ntl = base + tot;
    if (lane == 0) D.tl_n[t] = ntl;
    const int excl = inc - c.npend;
    for (int i = 0; i < c.npend; i++) {
        const int r = c.pend[i];
        const int k = base + excl + i;
        if (k >= LCAP) {
            set_err(D, E_CAPACITY, t, k, 3);
            continue;
        }
        Rec &R = D.rec[r];
        D.tl[(int64_t)t * LCAP + k] = r;
        if (R.x >= 0 && (R.flags & F_PEND)) {
            R.flags = F_LISTED;
            R.slot = k;
            D.tr[(int64_t)t * LCAP + k] = list_rate(R);
        } else {
            D.tr[(int64_t)t * LCAP + k] = 0.f;
        }
    }
    c.npend = 0;
    __syncwarp();
}

// Sites that neighbour tiles gave an event while this tile was idle join
// its list in grid-point order (a repeated record once); the inbox empties.
__device__ void drain_inbox(const Dev &D, int t, int lane, long long *key)
{
    const int m = min(D.ib_n[t], ICAP);
    if (m <= 0) return;
    const int32_t *in = D.ib + (int64_t)t * ICAP;
    const long long NONE = 0x7fffffffffffffffLL;
    for (int i = lane; i < m; i += 32) {
        const Rec &R = D.rec[in[i]];
        const bool ok = R.x >= 0 && tile_of(D, R.x, R.y) == t && (R.flags & F_INBOX) && R.ev != EV_NONE;
        key[i] = ok ? site_key(D, R) : NONE;
    }
    __syncwarp();
    // a repeated key keeps its first entry
    for (int i = lane; i < m; i += 32) {
        if (key[i] == NONE) continue;
        bool dup = false;
        for (int j = 0; j < i && !dup; j++) dup = key[j] == key[i];
        if (dup) key[i] = NONE - 1;
    }
    __syncwarp();
    int nv = 0;
    for (int i = lane; i < m; i += 32) nv += key[i] < NONE - 1;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) nv += __shfl_xor_sync(FULL, nv, o);
    const int base = D.tl_n[t];
    if (base + nv > LCAP) {
        if (lane == 0) set_err(D, E_CAPACITY, t, base + nv, 4);
        return;
    }
    for (int i = lane; i < m; i += 32) {
        const int r = in[i];
        Rec &R = D.rec[r];
        if (key[i] == NONE) {
            // lost its event (or moved, or freed) while waiting
            if (R.x >= 0 && tile_of(D, R.x, R.y) == t && (R.flags & F_INBOX)) R.flags = 0;
            continue;
        }
        if (key[i] == NONE - 1) continue;
        int rank = 0;
        for (int j = 0; j < m; j++) rank += key[j] < key[i];
        const int k = base + rank;
        R.flags = F_LISTED;
        R.slot = k;
        D.tl[(int64_t)t * LCAP + k] = r;
        D.tr[(int64_t)t * LCAP + k] = list_rate(R);
    }
    __syncwarp();
    if (lane == 0) {
        D.tl_n[t] = base + nv;
        D.ib_n[t] = 0;
    }
    __syncwarp();
}

// tile k of colour `colour` runs from the window's start to its end (one
// warp; every lane of the warp calls this)
__device__ void run_tile(const Dev &D, int colour, int k, uint32_t window, float tau)
{
    const int lane = threadIdx.x & 31;
    const int hx = D.ntx / 2;
    const int ti = 2 * (k % hx) + (colour & 1), tj = 2 * (k / hx) + (colour >> 1);
    const int t = tj * D.ntx + ti;
    int32_t *list = D.tl + (int64_t)t * LCAP;
    float *rates = D.tr + (int64_t)t * LCAP;
    // records freed in the tile's last phase become reusable
    if (lane == 0) {
        int np = min(D.fp_n[t], FCAP), nr = D.fr_n[t];
        for (int k = 0; k < np && nr < FCAP; k++) D.fr[(int64_t)t * FCAP + nr++] = D.fp[(int64_t)t * FCAP + k];
        D.fr_n[t] = nr;
        D.fp_n[t] = 0;
    }
    __syncwarp();
    {
        __shared__ long long inbox_key[4][ICAP];          // k_windows runs 4 warps per block
        drain_inbox(D, t, lane, inbox_key[(threadIdx.x >> 5) & 3]);
    }
    // compact the list once a quarter of it is dead.  An entry with a nonzero
    // rate is its record's current entry (a freed record's entry is zeroed,
    // and a record is appended again only after its entry was dropped); an
    // entry with rate 0 is kept only if it is the current entry (slot) of a
    // live record of this tile whose event has a zero rate, otherwise
    // dropped, and a record of this tile without an event whose current entry
    // it was may be listed again
    const int n = min(D.tl_n[t], LCAP);
    int dead = 0;
    for (int i = lane; i < n; i += 32) dead += rates[i] == 0.f;
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) dead += __shfl_xor_sync(FULL, dead, o);
    if (dead && (4 * dead > n || n > 3 * LCAP / 4)) {
        int out = 0;
        for (int base = 0; base < n; base += 32) {
            const int i = base + lane;
            int r = 0;
            float v = 0.f;
            bool keep = false;
            if (i < n) {
                r = list[i];
                v = rates[i];
                if (v != 0.f) {
                    keep = true;
                } else if (r > 0) {
                    Rec &R = D.rec[r];
                    const bool cur = R.x >= 0 && (R.flags & F_LISTED) && R.slot == i && tile_of(D, R.x, R.y) == t;
                    if (cur && R.ev != EV_NONE) keep = true;
                    else if (cur) R.flags &= (uint8_t)~F_LISTED;
                }
            }
            const unsigned km = __ballot_sync(FULL, keep);
            __syncwarp();
            if (keep) {
                const int pos = out + __popc(km & lanemask_lt());
                if (pos != i) {
                    list[pos] = r;
                    rates[pos] = v;
                    D.rec[r].slot = pos;
                }
            }
            out += __popc(km);
            __syncwarp();
        }
        if (lane == 0) D.tl_n[t] = out;
    }
    __syncwarp();

    Ctx c;
    c.tile = t;
    c.nbuff = P3{0, 0, 0};
    c.forced_arm = 0;
    c.key2 = window;
    c.key3 = 0x7a000000u | (uint32_t)colour;
    c.nties = 0;
    c.dmc = 0;
    c.npend = 0;
    float rem = tau;
    uint32_t nev = 0, ndraw = 0;
    int ntl = D.tl_n[t];                      // after drain and compaction (lane 0 wrote it before a __syncwarp)
    for (;;) {
        const int len = min(ntl, LCAP);
        // lane l owns the contiguous chunk [l C, l C + C) of the list: one
        // pass of independent loads gives each lane its partial sum, a warp
        // scan the prefix of every chunk
        const int C = (len + 31) >> 5;
        const int i0 = min(len, lane * C), i1 = min(len, i0 + C);
        float s = 0.f;
        int niso = 0;
        for (int i = i0; i < i1; i++) {
            const float v = rates[i];
            if (v > 0.f) s += v;
            else if (v < 0.f) niso++;
        }
        float inc = s;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            const float y = __shfl_up_sync(FULL, inc, o);
            if (lane >= o) inc += y;
        }
        float excl = __shfl_up_sync(FULL, inc, 1);
        if (lane == 0) excl = 0.f;
        const float tot = __shfl_sync(FULL, inc, 31);
        int nisot = niso;
#pragma unroll
        for (int o = 16; o > 0; o >>= 1) nisot += __shfl_xor_sync(FULL, nisot, o);
        // isolated atoms: 1e5 x the total rate (Get_Prob.f:305), the tile's here
        const float riso = nisot ? (float)nisot * 1.0e5f * fmaxf(tot, 1.0e-30f) : 0.f;
        const float rtot = tot + riso;
        if (!(rtot > 0.f)) break;
        U4 rnd = philox4x32_10(U4{ndraw++, (uint32_t)t, window, 0x51000000u | (uint32_t)colour}, D.k0, D.k1);
        float dt = -__logf(u01(rnd.x)) / rtot;
        if (dt > rem) break;
        rem -= dt;
        float target = u01(rnd.y) * rtot;
        int pick = -1;
        if (target >= tot && nisot > 0) {
            // the k-th isolated atom of the list
            int k = min((int)(u01(rnd.z) * (float)nisot), nisot - 1);
            for (int base = 0; base < len && pick < 0; base += 32) {
                int i = base + lane;
                const bool hit = i < len && rates[i] < 0.f;
                unsigned m = __ballot_sync(FULL, hit);
                if (k < __popc(m)) {
                    unsigned sel = __ballot_sync(FULL, hit && __popc(m & lanemask_lt()) == k);
                    pick = list[base + __ffs(sel) - 1];
                }
                k -= __popc(m);
            }
        } else {
            // the chunk whose prefix range holds the target, then its entry
            // (rounding at the top end: the last entry with a rate)
            const unsigned m = __ballot_sync(FULL, s > 0.f && inc > target);
            const unsigned nz = __ballot_sync(FULL, s > 0.f);
            if (nz) {
                const int L = m ? __ffs(m) - 1 : 31 - __clz(nz);
                int p = -1;
                if (lane == L) {
                    float acc = excl;
                    int lastnz = -1;
                    for (int i = i0; i < i1; i++) {
                        const float v = rates[i];
                        if (!(v > 0.f)) continue;
                        lastnz = i;
                        acc += v;
                        if (acc > target) break;
                    }
                    p = lastnz >= 0 ? list[lastnz] : -1;
                }
                pick = __shfl_sync(FULL, p, L);
            }
        }
        if (pick <= 0) break;
        __syncwarp();
        apply_warp(D, c, pick, u01(rnd.w), lane);
        flush_pending(D, c, t, lane, ntl);
        nev++;
        __syncwarp();
        if (block_err()) break;
    }
    if (lane == 0) {
        if (nev) atomicAdd(D.events, (unsigned long long)nev);
    }
    if (c.dmc) atomicAdd(D.nmc, c.dmc);          // every lane's own changes
}

// Grid-wide barrier of a cooperative launch (generation counter; all blocks
// are resident).  The wait is bounded: after `limit` cycles the block sets
// E_TIMEOUT and leaves, and every block sees the error after its own wait.
__device__ void grid_barrier(const Dev &D, unsigned *bar, long long limit)
{
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *gen = bar + 1;
        const unsigned g = *gen;
        __threadfence();
        if (atomicAdd(bar, 1u) + 1u == gridDim.x) {
            bar[0] = 0u;
            __threadfence();
            atomicAdd(bar + 1, 1u);
        } else {
            const long long t0 = clock64();
            while (*gen == g) {
                if (clock64() - t0 > limit) {
                    set_err(D, E_TIMEOUT, (int)blockIdx.x, 0, 0);
                    break;
                }
                __nanosleep(64);
            }
        }
        __threadfence();
    }
    __syncthreads();
}

// Persistent form: `nwin` windows from `w0`, the four colour phases of each
// separated by grid barriers; every warp takes the tiles wid, wid + W, ...
// of the colour.  At each window's start the replica stops once fewer than
// 21 sites keep an event (main.f:307-310) or `ev_limit` events are done.
__global__ void k_windows(Dev D, uint32_t w0, int nwin, float tau, unsigned long long ev_limit, unsigned *bar,
                          long long limit)
{
    const int wid = (int)((blockIdx.x * (unsigned)blockDim.x + threadIdx.x) >> 5);
    const int nw = (int)((gridDim.x * blockDim.x) >> 5);
    const int per = (D.ntx / 2) * (D.nty / 2);
    if (threadIdx.x == 0) s_block_err = 0;
    __syncthreads();
    for (int w = 0; w < nwin; w++) {
        if (*(volatile int32_t *)D.err || *(volatile int32_t *)D.stop) return;
        if (*(volatile int32_t *)D.nmc <= 20 || (ev_limit && *(volatile unsigned long long *)D.events >= ev_limit)) {
            grid_barrier(D, bar, limit);            // every block reads the counters before any sets stop
            if (blockIdx.x == 0 && threadIdx.x == 0) *D.stop = *(volatile int32_t *)D.nmc <= 20 ? 1 : 2;
            return;
        }
        for (int colour = 0; colour < 4; colour++) {
            for (int k = wid; k < per; k += nw) run_tile(D, colour, k, w0 + (uint32_t)w, tau);
            grid_barrier(D, bar, limit);
            if (*(volatile int32_t *)D.err) return;
        }
        if (blockIdx.x == 0 && threadIdx.x == 0) atomicAdd(D.windows_done, 1u);
    }
}

// the replay: events in order on one thread
__global__ void k_replay(Dev D, const mks_event *ev, long long n, long long *done)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    Ctx c;
    c.tile = -1;
    c.nbuff = P3{0, 0, 0};
    c.forced_arm = 0;
    c.key2 = c.key3 = 0;
    c.nties = 0;
    c.dmc = 0;
    c.npend = 0;
    long long k = 0;
    for (; k < n; k++) {
        const mks_event e = ev[k];
        P3 s{e.x, e.y, e.z};
        if (s.x < 0 || s.x >= D.lx || s.y < 0 || s.y >= D.ly || s.z < 0 || s.z > D.lz) {
            set_err(D, E_NOTAPPLICABLE, s.x, s.y, s.z);
            break;
        }
        const int64_t g = gidx(D, s);
        const uint32_t v = D.coo[g];
        const int r = D.ind[g];
        const uint8_t code = r > 0 ? D.rec[r].ev : EV_NONE;
        c.forced_arm = e.arm ? 1 : 0;
        if (e.itrans >= 1 && e.itrans <= 3) {
            if (occ_of(v) || (code != EV_DEP && code != EV_DUMMY) || (code == EV_DUMMY && e.itrans != 1)) {
                set_err(D, E_NOTAPPLICABLE, s.x, s.y, s.z);
                break;
            }
            deposition(D, c, s, e.itrans);
        } else if (e.itrans == 4) {
            if (!occ_of(v) || cov_of(v) == WALLIND || (code != EV_EVAP && code != EV_ISO)) {
                set_err(D, E_NOTAPPLICABLE, s.x, s.y, s.z);
                break;
            }
            evaporation(D, c, s);
        } else {
            set_err(D, E_NOTAPPLICABLE, s.x, s.y, s.z);
            break;
        }
        if (*(volatile int32_t *)D.err) {
            k++;
            break;
        }
    }
    *done = k;
    atomicAdd(D.nmc, c.dmc);
}

// rates of every record from the current lattice (Get_Prob_Ini.f:23-161: an
// empty coor-1 site marked ini keeps the init-time dummy rate 1e-6, :102-104),
// or, with gev / grate, the given event codes and rates kept as they are (the
// reference does not re-rate a site when only its neighbours' neighbours
// change, so a saved state's rates are not all what Get_Prob would give now);
// an evaporation whose site has no reciprocal neighbour is the isolated atom
// of Get_Prob.f:300-306 either way
__global__ void k_rate_all(Dev D, const uint8_t *ini, const int32_t *gev, const float *grate, int first, int last)
{
    for (int r = first + blockIdx.x * blockDim.x + threadIdx.x; r < last; r += gridDim.x * blockDim.x) {
        Rec &R = D.rec[r];
        if (R.x < 0) continue;
        P3 s{R.x, R.y, R.z};
        uint32_t v = cw(D, s);
        P3 nn[4];
        load_nn(R, nn);
        uint8_t ev = EV_NONE;
        float rate = 0.f;
        // a bulk atom (coordination 4) has no event and the reference never
        // asks Get_Prob about it: a slab without walls (SetSiCSF) leaves its
        // bottom layer at coordination 4 over empty sites
        if (!(occ_of(v) && coor_of(v) == 4)) get_prob(D, occ_of(v), sp_of(v), coor_of(v), s, nn, ev, rate);
        if (ev == EV_DUMMY && ini && ini[r]) rate = 1.e-6f;
        if (gev && ev != EV_ISO) {
            ev = (uint8_t)gev[r];
            rate = grate[r];
        }
        R.ev = ev;
        R.rate = rate;
        R.flags = 0;
    }
}

// tile lists from scratch, and the count of sites with an event
// Each tile's list in grid-point order after a rebuild (whose appends come
// in any order): a bitonic sort in shared memory, one block per tile.
__global__ void __launch_bounds__(256) k_sort_lists(Dev D)
{
    __shared__ long long key[LCAP];
    __shared__ int32_t id[LCAP];
    const int t = blockIdx.x;
    const int n = min(D.tl_n[t], LCAP);
    if (n < 2) return;
    int m = 1;
    while (m < n) m <<= 1;
    int32_t *list = D.tl + (int64_t)t * LCAP;
    for (int i = threadIdx.x; i < m; i += blockDim.x) {
        if (i < n) {
            id[i] = list[i];
            key[i] = site_key(D, D.rec[id[i]]);
        } else {
            id[i] = 0;
            key[i] = 0x7fffffffffffffffLL;
        }
    }
    __syncthreads();
    for (int k = 2; k <= m; k <<= 1)
        for (int j = k >> 1; j > 0; j >>= 1) {
            for (int i = threadIdx.x; i < m; i += blockDim.x) {
                const int p = i ^ j;
                if (p > i) {
                    const bool up = (i & k) == 0;
                    if ((key[i] > key[p]) == up) {
                        const long long tk = key[i];
                        key[i] = key[p];
                        key[p] = tk;
                        const int32_t ti = id[i];
                        id[i] = id[p];
                        id[p] = ti;
                    }
                }
            }
            __syncthreads();
        }
    for (int i = threadIdx.x; i < n; i += blockDim.x) {
        Rec &R = D.rec[id[i]];
        R.slot = i;
        list[i] = id[i];
        D.tr[(int64_t)t * LCAP + i] = list_rate(R);
    }
}

__global__ void k_rebuild(Dev D, int last)
{
    for (int r = 1 + blockIdx.x * blockDim.x + threadIdx.x; r < last; r += gridDim.x * blockDim.x) {
        Rec &R = D.rec[r];
        R.flags = 0;
        if (R.x < 0 || R.ev == EV_NONE) continue;
        atomicAdd(D.nmc, 1);
        int t = tile_of(D, R.x, R.y);
        int k = atomicAdd(&D.tl_n[t], 1);
        if (k >= LCAP) {
            set_err(D, E_CAPACITY, t, k, 1);
            continue;
        }
        R.flags = F_LISTED;
        R.slot = k;
        D.tl[(int64_t)t * LCAP + k] = r;
        D.tr[(int64_t)t * LCAP + k] = list_rate(R);
    }
}


// compact lattice -> LattCoo words and records.  Pass 1 counts the listed
// sites of each (z1, b) row; pass 2 writes them with ids from the row offsets.
__device__ __forceinline__ bool compact_site(int a, int b, int z1) { return ((a + b + (z1 >> 1)) & 1) == 0; }
__device__ __forceinline__ bool listed_byte(uint8_t s) { return s != 0 && s != 0x80 && ((s & 3) || ((s >> 2) & 7)); }

__global__ void k_count_rows(const uint8_t *st, int NA, int NB, int NZ, int pitch, int lz, int32_t *rowcnt)
{
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= NZ * NB) return;
    int z1 = row / NB, b = row % NB, k = 0;
    if (3 * z1 <= lz)
        for (int a = 0; a < NA; a++)
            if (compact_site(a, b, z1) && listed_byte(st[(int64_t)row * pitch + a])) k++;
    rowcnt[row] = k;
}

__global__ void k_expand(Dev D, const uint8_t *st, int NA, int NB, int NZ, int pitch, const int32_t *rowoff,
                         uint8_t *ini)
{
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= NZ * NB) return;
    const int z1 = row / NB, b = row % NB;
    const int z = 3 * z1;
    if (z > D.lz) return;
    int r = rowoff[row];
    const int zp = z1 & 1;
    for (int a = 0; a < NA; a++) {
        if (!compact_site(a, b, z1)) continue;
        uint8_t s = st[(int64_t)row * pitch + a];
        if (s == 0 || s == 0x80) continue;
        P3 p{3 * (2 * a + zp), 3 * (2 * b + zp), z};
        int sp = s & 3;
        int co = (s >> 2) & (7 ^ (s & 4));              // field 5 of an init-time dummy reads 1
        D.coo[gidx(D, p)] = ((uint32_t)co << 24) | (sp ? B_OCC : 0u) | ((uint32_t)sp << 27);
        if (!listed_byte(s)) continue;
        const int fd = (s >> 5) & 3;
        Rec &R = D.rec[r];
        R.x = (int16_t)p.x;
        R.y = (int16_t)p.y;
        R.z = (int16_t)p.z;
        // NextN: the four bonds (JumpDia order, defsystem.f:104-105) from the
        // first list entry on, as the initializers list them (SetSi.f:52-57);
        // an empty coor-1 site lists its one neighbour and zeros, as the
        // initializers' ad-void passes and deposition.f:86-99 write it
        const bool one = !sp && co == 1;
        for (int i = 0; i < 4; i++) {
            if (one && i > 0) {
                put_nn(R, i, P3{0, 0, 0});
                continue;
            }
            int d = (fd + i) & 3;
            int da = zp - (d >> 1), db = zp - ((d ^ (d >> 1)) & 1), dz = ((d ^ zp) & 1) ? -1 : 1;
            int aa = a + da, bb = b + db, kk = z1 + dz;
            P3 q{3 * (2 * aa + (kk & 1)), 3 * (2 * bb + (kk & 1)), 3 * kk};
            if (q.x < 0) q.x += D.lx;
            if (q.x >= D.lx) q.x -= D.lx;
            if (q.y < 0) q.y += D.ly;
            if (q.y >= D.ly) q.y -= D.ly;
            put_nn(R, i, q);
        }
        R.ev = EV_NONE;
        R.flags = 0;
        R.rate = 0.f;
        ini[r] = (s & 0x9C) == 0x94;                    // dummy flag with coordination field 5
        D.ind[gidx(D, p)] = r;
        r++;
    }
}

__global__ void k_wall_planes(Dev D, const int32_t *wall_plane)
{
    int64_t plane = (int64_t)D.lx * D.ly;
    int64_t nplanes = D.lz + 1;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < plane * nplanes;
         i += (int64_t)gridDim.x * blockDim.x) {
        int z = (int)(i / plane);
        if (wall_plane[z]) D.coo[(int64_t)(z + ZG) * plane + (i % plane)] = B_OCC | WALLIND;
    }
}

// per compact layer: sites, wall sites
__global__ void k_layer_walls(const uint8_t *st, int NA, int NB, int NZ, int pitch, int32_t *cnt)
{
    int row = blockIdx.x * blockDim.x + threadIdx.x;
    if (row >= NZ * NB) return;
    int z1 = row / NB, b = row % NB, ns = 0, nw = 0;
    for (int a = 0; a < NA; a++)
        if (compact_site(a, b, z1)) {
            ns++;
            nw += st[(int64_t)row * pitch + a] == 0x80;
        }
    atomicAdd(&cnt[2 * z1], ns);
    atomicAdd(&cnt[2 * z1 + 1], nw);
}

__global__ void k_load_records(Dev D, const int32_t *xyz, const int32_t *nn, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x) {
        Rec &R = D.rec[i + 1];
        P3 p{xyz[3 * i], xyz[3 * i + 1], xyz[3 * i + 2]};
        R.x = (int16_t)p.x;
        R.y = (int16_t)p.y;
        R.z = (int16_t)p.z;
        for (int k = 0; k < 4; k++) put_nn(R, k, P3{nn[12 * i + 3 * k], nn[12 * i + 3 * k + 1], nn[12 * i + 3 * k + 2]});
        R.ev = EV_NONE;
        R.flags = 0;
        R.rate = 0.f;
        D.ind[gidx(D, p)] = (int32_t)(i + 1);
    }
}

__global__ void k_gather(Dev D, int last, int32_t *word)
{
    for (int r = 1 + blockIdx.x * blockDim.x + threadIdx.x; r < last; r += gridDim.x * blockDim.x) {
        const Rec &R = D.rec[r];
        word[r] = R.x >= 0 ? (int32_t)cw(D, P3{R.x, R.y, R.z}) : 0;
    }
}

// FP32 rates of the sites whose event has a table rate (no dummy, no
// isolated atom), compacted into out
__global__ void k_event_rates(Dev D, int last, float *out, int32_t *cnt)
{
    for (int r = 1 + blockIdx.x * blockDim.x + threadIdx.x; r < last; r += gridDim.x * blockDim.x) {
        const Rec &R = D.rec[r];
        if (R.x < 0 || (R.ev != EV_DEP && R.ev != EV_EVAP) || !(R.rate > 0.f)) continue;
        out[atomicAdd(cnt, 1)] = R.rate;
    }
}

// the reference's diamond-site test (SetSi.f:52-57)
__device__ __forceinline__ bool dia_site(int x, int y, int z)
{
    if (x % 3 || y % 3 || z % 3) return false;
    int x1 = x / 3, y1 = y / 3, z1 = z / 3;
    if ((x1 & 1) != (y1 & 1) || (x1 & 1) != (z1 & 1)) return false;
    int m = (x1 + y1 + z1) & 3;
    return m == 0 || m == 3;
}

// counters: 0 atoms, 1 undercoordinated, 2 with an event, 3 voids, 4..6
// species, 7 non-epitaxial bulk; rate sums [0] non-isolated, [1] isolated
// count; column tops (6 x 6 grid-unit columns)
__global__ void k_observe(Dev D, int last, unsigned long long *cnt, double *rsum, int32_t *coltop)
{
    __shared__ unsigned long long sc[8];
    __shared__ double sr[2];
    if (threadIdx.x < 8) sc[threadIdx.x] = 0;
    if (threadIdx.x < 2) sr[threadIdx.x] = 0.0;
    __syncthreads();
    const int ncx = D.lx / 6;
    for (int r = 1 + blockIdx.x * blockDim.x + threadIdx.x; r < last; r += gridDim.x * blockDim.x) {
        const Rec &R = D.rec[r];
        if (R.x < 0) continue;
        uint32_t v = cw(D, P3{R.x, R.y, R.z});
        if (R.ev != EV_NONE) {
            atomicAdd(&sc[2], 1ull);
            if (R.ev == EV_ISO) atomicAdd(&sr[1], 1.0);
            else atomicAdd(&sr[0], (double)R.rate);
        }
        if (occ_of(v) && cov_of(v) != WALLIND) {
            atomicAdd(&sc[0], 1ull);
            int co = coor_of(v), s = sp_of(v);
            if (co <= 3) atomicAdd(&sc[1], 1ull);
            if (s >= 1 && s <= 3) atomicAdd(&sc[3 + s], 1ull);
            if (co == 4 && R.z >= 0 && R.z < D.lz && !dia_site(R.x, R.y, R.z)) atomicAdd(&sc[7], 1ull);
            atomicMax(&coltop[(R.y / 6) * ncx + R.x / 6], (int)R.z);
        } else if (!occ_of(v) && coor_of(v) == 4) {
            atomicAdd(&sc[3], 1ull);
        }
    }
    __syncthreads();
    if (threadIdx.x < 8) atomicAdd(&cnt[threadIdx.x], sc[threadIdx.x]);
    if (threadIdx.x < 2) atomicAdd(&rsum[threadIdx.x], sr[threadIdx.x]);
}

int grid_for(int64_t n, int block = 256) { return (int)std::max<int64_t>(1, std::min<int64_t>(152 * 32, (n + block - 1) / block)); }

}  // namespace

struct State {
    mks_config cfg{};
    cudaStream_t stream = nullptr;
    Dev D{};
    int64_t ngrid = 0;
    int nrec = 0;                 // records in use at load (ids 1..nrec)
    double ptransE[3 * 4096] = {0}, ptransD[9] = {0};
    bool rates = false, ready = false, lists_ok = false;
    double time = 0.0;
    int64_t window = 0, events = 0;
    int32_t *d_scratch = nullptr;
    unsigned *d_bar = nullptr;   // grid barrier of the persistent kernel (count, generation)
    double *d_tab = nullptr;
    float *d_tabf = nullptr;
    int stop_reason = 0;
    int last_error = 0;
};

namespace {

int ferr(std::string &err, int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    err = buf;
    return code;
}

#define SK(call)                                                                                      \
    do {                                                                                              \
        cudaError_t e_ = (call);                                                                      \
        if (e_ != cudaSuccess) return ferr(err, MKS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

int upload_tables(State *s, std::string &err)
{
    double tab[192 + 9];
    float tf[192 + 9];
    for (int sp = 0; sp < 3; sp++)
        for (int n1 = 0; n1 < 4; n1++)
            for (int n2 = 0; n2 < 4; n2++)
                for (int n3 = 0; n3 < 4; n3++)
                    tab[sp * 64 + n1 * 16 + n2 * 4 + n3] = s->ptransE[sp * 4096 + n1 * 1024 + n2 * 256 + n3 * 64];
    for (int k = 0; k < 9; k++) tab[192 + k] = s->ptransD[k];
    for (int k = 0; k < 192; k++) tf[k] = (float)tab[k];
    for (int co = 1; co <= 3; co++) {
        // Get_Prob.f:159-176: the deposition rate is the FP64 sum over species
        const double p1 = s->ptransD[co - 1], p2 = s->ptransD[3 + co - 1], p3 = s->ptransD[6 + co - 1];
        const double tot = p1 + p2 + p3;
        tf[192 + co - 1] = (float)tot;
        tf[195 + 2 * (co - 1)] = tot > 0 ? (float)(p1 / tot) : 1.f;
        tf[196 + 2 * (co - 1)] = tot > 0 ? (float)((p1 + p2) / tot) : 1.f;
    }
    SK(cudaMemcpyAsync(s->d_tab, tab, sizeof tab, cudaMemcpyHostToDevice, s->stream));
    SK(cudaMemcpyAsync(s->d_tabf, tf, sizeof tf, cudaMemcpyHostToDevice, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    return 0;
}

const char *derr_name(int code)
{
    switch (code) {
    case E_INVARIANT: return "lattice state contradicts the model";
    case E_CAPACITY: return "a tile list or the record pool is full";
    case E_NOTAPPLICABLE: return "event not applicable to the lattice state";
    case E_BOUNDS: return "grid point outside the box";
    case E_NBUFF: return "no occupied neighbour lists the site (stale NBuff)";
    case E_ARM: return "stacking choice differs from the trace";
    case E_TIMEOUT: return "a block waited too long at the grid barrier";
    default: return "device error";
    }
}

int check_device(State *s, std::string &err, const char *what)
{
    int32_t e[4];
    SK(cudaMemcpyAsync(e, s->D.err, sizeof e, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    if (!e[0]) return 0;
    SK(cudaMemsetAsync(s->D.err, 0, 4 * sizeof(int32_t), s->stream));
    SK(cudaStreamSynchronize(s->stream));
    s->last_error = e[0];
    int code = e[0] == E_CAPACITY ? MKS_ERR_CAPACITY
             : e[0] == E_TIMEOUT ? MKS_ERR_TIMEOUT
             : (e[0] == E_NOTAPPLICABLE || e[0] == E_ARM) ? MKS_ERR_ARG : MKS_ERR_INVARIANT;
    return ferr(err, code, "%s: %s at (%d, %d, %d)", what, derr_name(e[0]), e[1], e[2], e[3]);
}

int rates_and_lists(State *s, const uint8_t *d_ini, std::string &err, const int32_t *d_ev = nullptr,
                    const float *d_rate = nullptr)
{
    int top = s->nrec + 1;
    SK(cudaMemcpyAsync(s->D.top, &top, sizeof top, cudaMemcpyHostToDevice, s->stream));
    if (top > 1) k_rate_all<<<grid_for(top), 256, 0, s->stream>>>(s->D, d_ini, d_ev, d_rate, 1, top);
    SK(cudaGetLastError());
    int ntiles = s->D.ntx * s->D.nty;
    SK(cudaMemsetAsync(s->D.fr_n, 0, sizeof(int32_t) * ntiles, s->stream));
    SK(cudaMemsetAsync(s->D.fp_n, 0, sizeof(int32_t) * ntiles, s->stream));
    s->lists_ok = false;
    s->ready = true;
    return check_device(s, err, "rates");
}

int rebuild(State *s, std::string &err)
{
    int top = 0;
    SK(cudaMemcpyAsync(&top, s->D.top, sizeof top, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    int ntiles = s->D.ntx * s->D.nty;
    SK(cudaMemsetAsync(s->D.tl_n, 0, sizeof(int32_t) * ntiles, s->stream));
    SK(cudaMemsetAsync(s->D.nmc, 0, sizeof(int32_t), s->stream));
    SK(cudaMemsetAsync(s->D.ib_n, 0, sizeof(int32_t) * ntiles, s->stream));
    if (top > 1) k_rebuild<<<grid_for(top), 256, 0, s->stream>>>(s->D, top);
    k_sort_lists<<<ntiles, 256, 0, s->stream>>>(s->D);
    SK(cudaGetLastError());
    s->lists_ok = true;
    return check_device(s, err, "list build");
}

}  // namespace

int create(State **out, const mks_config &cfg, cudaStream_t stream, std::string &err)
{
    *out = nullptr;
    const int lx = cfg.lenx, ly = cfg.leny, lz = cfg.lenz;
    if (lx > 30000 || ly > 30000 || lz + ZG > 30000)
        return ferr(err, MKS_ERR_ARG, "box %dx%dx%d: sides up to 30000 grid units with arm-chair stacking", lx, ly, lz);
    if (cfg.ncov != 0) return ferr(err, MKS_ERR_UNSUPPORTED, "arm-chair stacking with a coverage species");
    if (!(cfg.ptrans_zig >= 0.0 && cfg.ptrans_zig <= 1.0))
        return ferr(err, MKS_ERR_ARG, "PtransZig=%g outside [0, 1]", cfg.ptrans_zig);
    // an even number of tiles per side, each at least TWMIN wide
    auto tiles = [](int L) {
        for (int n = L / TWMIN; n >= 2; n--)
            if (n % 2 == 0 && L % n == 0) return n;
        return 0;
    };
    int ntx = tiles(lx), nty = tiles(ly);
    if (!ntx || !nty)
        return ferr(err, MKS_ERR_ARG, "box %dx%d cannot be cut into an even number of tiles >= %d grid units wide",
                    lx, ly, TWMIN);
    if (lx / ntx != ly / nty)
        return ferr(err, MKS_ERR_ARG, "box %dx%d: square tiles need LenX/ntiles = LenY/ntiles", lx, ly);
    State *s = new State;
    s->cfg = cfg;
    s->stream = stream;
    Dev &D = s->D;
    D.lx = lx;
    D.ly = ly;
    D.lz = lz;
    D.ntx = ntx;
    D.nty = nty;
    D.tw = lx / ntx;
    s->ngrid = (int64_t)(lz + 1 + 2 * ZG) * ly * lx;
    int ntiles = ntx * nty;
    // records: every diamond site of the box could be listed, and growth
    // adds sites beyond them; 25 % headroom above the site count
    int64_t sites = (int64_t)lx * ly * (lz + 1) / 216 * 8 / 4 + 1;
    int64_t rcap = std::min<int64_t>(INT32_MAX - 1, sites + sites / 4 + (1 << 20));
    D.rcap = (int)rcap;
    const double pi = (double)3.14159265358979323f;   // FIND_NN.f:37: default-REAL literal
    for (int irot = 1; irot <= 2; irot++) {
        D.cth[irot - 1] = cos((double)(2 * irot) * pi / 3.0);
        D.sth[irot - 1] = sin((double)(2 * irot) * pi / 3.0);
    }
    D.shift = (double)8.6602254037f;                  // FIND_SN.f:67
    D.pzig = cfg.ptrans_zig;
    D.k0 = (uint32_t)cfg.seed;
    D.k1 = (uint32_t)(cfg.seed >> 32) ^ 0xa511e9b3u;
    auto fail_free = [&](int rc) {
        destroy(s);
        return rc;
    };
#define SA(p, bytes)                                                                         \
    do {                                                                                     \
        cudaError_t e_ = cudaMalloc((void **)&(p), (bytes));                                 \
        if (e_ != cudaSuccess) {                                                             \
            ferr(err, MKS_ERR_CUDA, "cudaMalloc %lld bytes: %s", (long long)(bytes), cudaGetErrorString(e_)); \
            return fail_free(MKS_ERR_CUDA);                                                  \
        }                                                                                    \
    } while (0)
    SA(D.coo, sizeof(uint32_t) * s->ngrid);
    SA(D.ind, sizeof(int32_t) * s->ngrid);
    SA(D.rec, sizeof(Rec) * (size_t)rcap);
    SA(D.tl, sizeof(int32_t) * (size_t)ntiles * LCAP);
    SA(D.tr, sizeof(float) * (size_t)ntiles * LCAP);
    SA(D.ib, sizeof(int32_t) * (size_t)ntiles * ICAP);
    SA(D.ib_n, sizeof(int32_t) * ntiles);
    SA(D.tl_n, sizeof(int32_t) * ntiles);
    SA(D.fr, sizeof(int32_t) * (size_t)ntiles * FCAP);
    SA(D.fr_n, sizeof(int32_t) * ntiles);
    SA(D.fp, sizeof(int32_t) * (size_t)ntiles * FCAP);
    SA(D.fp_n, sizeof(int32_t) * ntiles);
    SA(s->d_scratch, sizeof(int32_t) * 16 + sizeof(unsigned long long) * 2);
    SA(s->d_tab, sizeof(double) * (192 + 9));
    SA(s->d_tabf, sizeof(float) * (192 + 9));
#undef SA
    int32_t *sc = s->d_scratch;
    D.err = sc;                 // 4
    D.nmc = sc + 4;
    D.stop = sc + 5;
    D.top = sc + 6;
    D.events = reinterpret_cast<unsigned long long *>(sc + 8);
    D.windows_done = reinterpret_cast<unsigned *>(sc + 12);
    s->d_bar = reinterpret_cast<unsigned *>(sc + 13);     // 2 words
    D.pe = s->d_tab;
    D.pd = s->d_tab + 192;
    D.pef = s->d_tabf;
    D.pds = s->d_tabf + 192;
    cudaError_t e = cudaMemsetAsync(s->d_scratch, 0, sizeof(int32_t) * 16 + sizeof(unsigned long long) * 2, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(D.coo, 0, sizeof(uint32_t) * s->ngrid, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(D.ind, 0, sizeof(int32_t) * s->ngrid, stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(D.rec, 0, sizeof(Rec), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_tab, 0, sizeof(double) * (192 + 9), stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(s->d_tabf, 0, sizeof(float) * (192 + 9), stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(stream);
    if (e != cudaSuccess) {
        ferr(err, MKS_ERR_CUDA, "clearing the lattice: %s", cudaGetErrorString(e));
        return fail_free(MKS_ERR_CUDA);
    }
    *out = s;
    return 0;
}

void destroy(State *s)
{
    if (!s) return;
    Dev &D = s->D;
    cudaFree(D.coo);
    cudaFree(D.ind);
    cudaFree(D.rec);
    cudaFree(D.tl);
    cudaFree(D.tr);
    cudaFree(D.ib);
    cudaFree(D.ib_n);
    cudaFree(D.tl_n);
    cudaFree(D.fr);
    cudaFree(D.fr_n);
    cudaFree(D.fp);
    cudaFree(D.fp_n);
    cudaFree(s->d_scratch);
    cudaFree(s->d_tab);
    cudaFree(s->d_tabf);
    delete s;
}

bool loaded(const State *s) { return s && s->ready; }

int set_rates(State *s, const double *ptransE, const double *ptransD, std::string &err)
{
    memcpy(s->ptransE, ptransE, sizeof s->ptransE);
    memcpy(s->ptransD, ptransD, sizeof s->ptransD);
    s->rates = true;
    int rc = upload_tables(s, err);
    if (rc) return rc;
    if (s->ready) {   // re-rate the current lattice (SetProbability then Get_Prob of every site)
        int top = 0;
        SK(cudaMemcpyAsync(&top, s->D.top, sizeof top, cudaMemcpyDeviceToHost, s->stream));
        SK(cudaStreamSynchronize(s->stream));
        if (top > 1) k_rate_all<<<grid_for(top), 256, 0, s->stream>>>(s->D, nullptr, nullptr, nullptr, 1, top);
        SK(cudaGetLastError());
        s->lists_ok = false;
        return check_device(s, err, "rates");
    }
    return 0;
}

int from_compact(State *s, const uint8_t *d_st, int NA, int NB, int NZ, int pitch, std::string &err)
{
    Dev &D = s->D;
    if (NA * 6 != D.lx || NB * 6 != D.ly) return ferr(err, MKS_ERR_ARG, "compact lattice does not match the box");
    const int rows = NZ * NB;
    SK(cudaMemsetAsync(D.coo, 0, sizeof(uint32_t) * s->ngrid, s->stream));
    SK(cudaMemsetAsync(D.ind, 0, sizeof(int32_t) * s->ngrid, s->stream));
    int32_t *d_rows = nullptr, *d_lw = nullptr;
    uint8_t *d_ini = nullptr;
    SK(cudaMallocAsync(&d_rows, sizeof(int32_t) * rows, s->stream));
    SK(cudaMallocAsync(&d_lw, sizeof(int32_t) * 2 * NZ, s->stream));
    SK(cudaMemsetAsync(d_lw, 0, sizeof(int32_t) * 2 * NZ, s->stream));
    k_count_rows<<<(rows + 127) / 128, 128, 0, s->stream>>>(d_st, NA, NB, NZ, pitch, D.lz, d_rows);
    k_layer_walls<<<(rows + 127) / 128, 128, 0, s->stream>>>(d_st, NA, NB, NZ, pitch, d_lw);
    SK(cudaGetLastError());
    std::vector<int32_t> rc(rows), lw(2 * NZ);
    SK(cudaMemcpyAsync(rc.data(), d_rows, sizeof(int32_t) * rows, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaMemcpyAsync(lw.data(), d_lw, sizeof(int32_t) * 2 * NZ, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    // walls: a layer of wall sites stands for its three grid planes, every
    // grid point of them a wall (SetSi.f:38-46,212-220); a layer with only
    // some wall sites has wall points off the diamond sub-grid that the
    // compact lattice does not record
    std::vector<int32_t> wp(D.lz + 1, 0);
    for (int z1 = 0; z1 < NZ; z1++) {
        if (lw[2 * z1 + 1] == 0) continue;
        if (lw[2 * z1 + 1] != lw[2 * z1]) {
            cudaFreeAsync(d_rows, s->stream);
            cudaFreeAsync(d_lw, s->stream);
            return ferr(err, MKS_ERR_UNSUPPORTED,
                        "layer z=%d holds a partial wall block: its points off the diamond sites are not in the "
                        "compact lattice (arm-chair stacking needs them)", 3 * z1);
        }
        for (int zz = 3 * z1; zz < 3 * z1 + 3 && zz <= D.lz; zz++) wp[zz] = 1;
    }
    std::vector<int32_t> off(rows);
    int64_t tot = 0;
    for (int i = 0; i < rows; i++) {
        off[i] = (int32_t)(tot + 1);
        tot += rc[i];
    }
    if (tot + 1 > D.rcap) {
        cudaFreeAsync(d_rows, s->stream);
        cudaFreeAsync(d_lw, s->stream);
        return ferr(err, MKS_ERR_CAPACITY, "%lld listed sites exceed the record pool", (long long)tot);
    }
    SK(cudaMemcpyAsync(d_rows, off.data(), sizeof(int32_t) * rows, cudaMemcpyHostToDevice, s->stream));
    SK(cudaMallocAsync(&d_ini, (size_t)tot + 2, s->stream));
    SK(cudaMemsetAsync(d_ini, 0, (size_t)tot + 2, s->stream));
    int32_t *d_wplanes = nullptr;
    SK(cudaMallocAsync(&d_wplanes, sizeof(int32_t) * (D.lz + 1), s->stream));
    SK(cudaMemcpyAsync(d_wplanes, wp.data(), sizeof(int32_t) * (D.lz + 1), cudaMemcpyHostToDevice, s->stream));
    k_wall_planes<<<grid_for((int64_t)D.lx * D.ly * (D.lz + 1)), 256, 0, s->stream>>>(D, d_wplanes);
    k_expand<<<(rows + 127) / 128, 128, 0, s->stream>>>(D, d_st, NA, NB, NZ, pitch, d_rows, d_ini);
    SK(cudaGetLastError());
    s->nrec = (int)tot;
    int r = rates_and_lists(s, d_ini, err);
    cudaFreeAsync(d_rows, s->stream);
    cudaFreeAsync(d_lw, s->stream);
    cudaFreeAsync(d_ini, s->stream);
    cudaFreeAsync(d_wplanes, s->stream);
    SK(cudaStreamSynchronize(s->stream));
    s->time = 0.0;
    s->window = 0;
    s->events = 0;
    s->stop_reason = 0;
    return r;
}

int load_lists(State *s, const int32_t *lattcoo, int64_t n, const int32_t *xyz, const int32_t *nn,
               const int32_t *event, const float *rate, std::string &err)
{
    Dev &D = s->D;
    if (n + 1 > D.rcap) return ferr(err, MKS_ERR_CAPACITY, "%lld list entries exceed the record pool", (long long)n);
    for (int64_t i = 0; i < n; i++) {
        const int32_t *p = xyz + 3 * i;
        if (p[0] < 0 || p[0] >= D.lx || p[1] < 0 || p[1] >= D.ly || p[2] < 0 || p[2] > D.lz)
            return ferr(err, MKS_ERR_ARG, "list entry %lld at (%d, %d, %d) is outside the box", (long long)i, p[0], p[1],
                        p[2]);
        for (int k = 0; k < 4; k++) {
            const int32_t *q = nn + 12 * i + 3 * k;
            if (q[0] < 0 || q[0] >= D.lx || q[1] < 0 || q[1] >= D.ly || q[2] < -ZG || q[2] > D.lz + ZG)
                return ferr(err, MKS_ERR_ARG, "NextN %d of list entry %lld is outside the box", k, (long long)i);
        }
    }
    const int64_t plane = (int64_t)D.lx * D.ly;
    SK(cudaMemsetAsync(D.coo, 0, sizeof(uint32_t) * s->ngrid, s->stream));
    SK(cudaMemsetAsync(D.ind, 0, sizeof(int32_t) * s->ngrid, s->stream));
    SK(cudaMemcpyAsync(D.coo + ZG * plane, lattcoo, sizeof(int32_t) * plane * (D.lz + 1), cudaMemcpyHostToDevice,
                       s->stream));
    if (event)
        for (int64_t i = 0; i < n; i++)
            if (event[i] != EV_NONE && event[i] != EV_DEP && event[i] != EV_DUMMY && event[i] != EV_EVAP &&
                event[i] != EV_ISO)
                return ferr(err, MKS_ERR_ARG, "event code %d of list entry %lld", event[i], (long long)i);
    int32_t *d_xyz = nullptr, *d_nn = nullptr, *d_ev = nullptr;
    float *d_rate = nullptr;
    uint8_t *d_ini = nullptr;
    size_t nb = (size_t)std::max<int64_t>(n, 1);
    SK(cudaMallocAsync(&d_xyz, sizeof(int32_t) * 3 * nb, s->stream));
    SK(cudaMallocAsync(&d_nn, sizeof(int32_t) * 12 * nb, s->stream));
    SK(cudaMallocAsync(&d_ini, nb + 2, s->stream));
    SK(cudaMemsetAsync(d_ini, 1, nb + 2, s->stream));   // loading is an initialization: Get_Prob_Ini's dummy rate
    if (event && rate) {
        SK(cudaMallocAsync(&d_ev, sizeof(int32_t) * (nb + 1), s->stream));
        SK(cudaMallocAsync(&d_rate, sizeof(float) * (nb + 1), s->stream));
    }
    if (n) {
        SK(cudaMemcpyAsync(d_xyz, xyz, sizeof(int32_t) * 3 * n, cudaMemcpyHostToDevice, s->stream));
        SK(cudaMemcpyAsync(d_nn, nn, sizeof(int32_t) * 12 * n, cudaMemcpyHostToDevice, s->stream));
        if (d_ev) {
            SK(cudaMemcpyAsync(d_ev + 1, event, sizeof(int32_t) * n, cudaMemcpyHostToDevice, s->stream));
            SK(cudaMemcpyAsync(d_rate + 1, rate, sizeof(float) * n, cudaMemcpyHostToDevice, s->stream));
        }
        k_load_records<<<grid_for(n), 256, 0, s->stream>>>(D, d_xyz, d_nn, (long long)n);
        SK(cudaGetLastError());
    }
    s->nrec = (int)n;
    int r = rates_and_lists(s, d_ini, err, d_ev, d_rate);
    cudaFreeAsync(d_xyz, s->stream);
    cudaFreeAsync(d_nn, s->stream);
    cudaFreeAsync(d_ini, s->stream);
    if (d_ev) cudaFreeAsync(d_ev, s->stream);
    if (d_rate) cudaFreeAsync(d_rate, s->stream);
    SK(cudaStreamSynchronize(s->stream));
    s->time = 0.0;
    s->window = 0;
    s->events = 0;
    s->stop_reason = 0;
    return r;
}

int replay(State *s, const mks_event *trace, int64_t n, int64_t *done, std::string &err)
{
    if (!s->ready) return ferr(err, MKS_ERR_ARG, "no lattice loaded");
    if (done) *done = 0;
    if (n <= 0) return 0;
    mks_event *d_ev = nullptr;
    long long *d_done = nullptr;
    SK(cudaMallocAsync(&d_ev, sizeof(mks_event) * (size_t)n, s->stream));
    SK(cudaMallocAsync(&d_done, sizeof(long long), s->stream));
    SK(cudaMemcpyAsync(d_ev, trace, sizeof(mks_event) * (size_t)n, cudaMemcpyHostToDevice, s->stream));
    SK(cudaMemsetAsync(s->D.fr_n, 0, sizeof(int32_t), s->stream));
    k_replay<<<1, 32, 0, s->stream>>>(s->D, d_ev, (long long)n, d_done);
    SK(cudaGetLastError());
    long long k = 0;
    SK(cudaMemcpyAsync(&k, d_done, sizeof k, cudaMemcpyDeviceToHost, s->stream));
    cudaFreeAsync(d_ev, s->stream);
    cudaFreeAsync(d_done, s->stream);
    SK(cudaStreamSynchronize(s->stream));
    SK(cudaMemsetAsync(s->D.fr_n, 0, sizeof(int32_t), s->stream));
    if (done) *done = k;
    s->events += k;
    s->lists_ok = false;
    return check_device(s, err, "replay");
}

int run(State *s, double tau, int64_t max_windows, int64_t max_events, double max_time, int64_t *events,
        double *time, std::string &err)
{
    if (!s->ready) return ferr(err, MKS_ERR_ARG, "no lattice loaded");
    if (!s->rates) return ferr(err, MKS_ERR_ARG, "rates not set");
    if (!(tau > 0.0)) return ferr(err, MKS_ERR_ARG, "tau must be positive");
    if (!s->lists_ok) {
        int rc = rebuild(s, err);
        if (rc) return rc;
    }
    Dev &D = s->D;
    unsigned long long e0 = 0;
    SK(cudaMemcpyAsync(&e0, D.events, sizeof e0, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaMemsetAsync(D.stop, 0, sizeof(int32_t), s->stream));
    SK(cudaStreamSynchronize(s->stream));
    s->stop_reason = 0;
    // one cooperative launch per block of windows: every block resident, the
    // warps striding over the tiles of each colour
    const int per = (D.ntx / 2) * (D.nty / 2);
    int dev = 0, nsm = 0, per_sm = 0;
    SK(cudaGetDevice(&dev));
    SK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    SK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_windows, 128, 0));
    if (per_sm < 1) return ferr(err, MKS_ERR_CUDA, "the window kernel cannot be resident");
    const int blocks = (int)std::min<int64_t>((int64_t)(per * 32 + 127) / 128, (int64_t)nsm * per_sm);
    const long long limit = 4000000000LL;        // cycles a block waits at a barrier (about 2 s)
    int64_t w = 0;
    const int64_t batch = 64;
    unsigned long long ev = e0;
    while (max_windows <= 0 || w < max_windows) {
        int64_t nb = max_windows > 0 ? std::min<int64_t>(batch, max_windows - w) : batch;
        if (max_time > 0.0) {
            int64_t left = s->time < max_time ? std::max<int64_t>(1, (int64_t)ceil((max_time - s->time) / tau)) : 0;
            if (left <= 0) {
                s->stop_reason = 3;
                break;
            }
            nb = std::min(nb, left);
        }
        SK(cudaMemsetAsync(s->d_bar, 0, 2 * sizeof(unsigned), s->stream));
        SK(cudaMemsetAsync(D.windows_done, 0, sizeof(unsigned), s->stream));
        uint32_t w0 = (uint32_t)s->window;
        int nwin = (int)nb;
        float ftau = (float)tau;
        unsigned long long ev_limit = max_events > 0 ? e0 + (unsigned long long)max_events : 0ull;
        unsigned *bar = s->d_bar;
        long long lim = limit;
        void *args[] = {&D, &w0, &nwin, &ftau, &ev_limit, &bar, &lim};
        SK(cudaLaunchCooperativeKernel((const void *)k_windows, dim3(blocks), dim3(128), args, 0, s->stream));
        int rc = check_device(s, err, "run");
        if (rc) {
            s->lists_ok = false;
            return rc;
        }
        int32_t stop = 0;
        unsigned done = 0;
        SK(cudaMemcpyAsync(&ev, D.events, sizeof ev, cudaMemcpyDeviceToHost, s->stream));
        SK(cudaMemcpyAsync(&stop, D.stop, sizeof stop, cudaMemcpyDeviceToHost, s->stream));
        SK(cudaMemcpyAsync(&done, D.windows_done, sizeof done, cudaMemcpyDeviceToHost, s->stream));
        SK(cudaStreamSynchronize(s->stream));
        s->window += done;
        s->time += (double)done * tau;
        w += done;
        if (stop) {
            s->stop_reason = stop == 1 ? 1 : 2;
            break;
        }
    }
    s->events += (int64_t)(ev - e0);
    if (events) *events = (int64_t)(ev - e0);
    if (time) *time = s->time;
    return 0;
}

int get_lattice(State *s, int32_t *lattcoo, std::string &err)
{
    const int64_t plane = (int64_t)s->D.lx * s->D.ly;
    SK(cudaMemcpyAsync(lattcoo, s->D.coo + ZG * plane, sizeof(int32_t) * plane * (s->D.lz + 1), cudaMemcpyDeviceToHost,
                       s->stream));
    SK(cudaStreamSynchronize(s->stream));
    return 0;
}

int sites(State *s, std::vector<Site> &out, std::string &err)
{
    out.clear();
    int top = 0;
    SK(cudaMemcpyAsync(&top, s->D.top, sizeof top, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    std::vector<Rec> rec((size_t)std::max(top, 1));
    std::vector<int32_t> word((size_t)std::max(top, 1));
    int32_t *d_word = nullptr;
    SK(cudaMallocAsync(&d_word, sizeof(int32_t) * (size_t)std::max(top, 1), s->stream));
    if (top > 1) k_gather<<<grid_for(top), 256, 0, s->stream>>>(s->D, top, d_word);
    SK(cudaGetLastError());
    SK(cudaMemcpyAsync(rec.data(), s->D.rec, sizeof(Rec) * (size_t)top, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaMemcpyAsync(word.data(), d_word, sizeof(int32_t) * (size_t)top, cudaMemcpyDeviceToHost, s->stream));
    cudaFreeAsync(d_word, s->stream);
    SK(cudaStreamSynchronize(s->stream));
    for (int r = 1; r < top; r++) {
        const Rec &R = rec[r];
        if (R.x < 0) continue;
        Site t;
        t.x = R.x;
        t.y = R.y;
        t.z = R.z;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 3; j++) t.nn[i][j] = R.nn[i][j];
        t.word = (uint32_t)word[r];
        t.ev = R.ev;
        t.rate = R.rate;
        out.push_back(t);
    }
    return 0;
}

int event_rates(State *s, std::vector<float> &out, std::string &err)
{
    out.clear();
    int top = 0;
    SK(cudaMemcpyAsync(&top, s->D.top, sizeof top, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    if (top <= 1) return 0;
    float *d_out = nullptr;
    int32_t *d_cnt = nullptr;
    SK(cudaMallocAsync(&d_out, sizeof(float) * (size_t)top, s->stream));
    SK(cudaMallocAsync(&d_cnt, sizeof(int32_t), s->stream));
    SK(cudaMemsetAsync(d_cnt, 0, sizeof(int32_t), s->stream));
    k_event_rates<<<grid_for(top), 256, 0, s->stream>>>(s->D, top, d_out, d_cnt);
    SK(cudaGetLastError());
    int32_t n = 0;
    SK(cudaMemcpyAsync(&n, d_cnt, sizeof n, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    out.resize((size_t)n);
    if (n) SK(cudaMemcpyAsync(out.data(), d_out, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, s->stream));
    cudaFreeAsync(d_out, s->stream);
    cudaFreeAsync(d_cnt, s->stream);
    SK(cudaStreamSynchronize(s->stream));
    return 0;
}

int get_lists(State *s, int64_t cap, int32_t *xyz, int32_t *nn, int32_t *kind, int32_t *evc, float *rate,
              int64_t *n, std::string &err)
{
    std::vector<Site> all;
    int rc = sites(s, all, err);
    if (rc) return rc;
    *n = (int64_t)all.size();
    if (!(xyz && nn && kind && evc && rate) || cap < *n) return 0;
    for (size_t k = 0; k < all.size(); k++) {
        const Site &t = all[k];
        uint32_t v = t.word;
        int kd = t.ev ? 1 : (((v >> 23) & 1) && ((v >> 24) & 7) == 4 ? 2 : (((v >> 24) & 7) == 4 ? 3 : 0));
        xyz[3 * k] = t.x;
        xyz[3 * k + 1] = t.y;
        xyz[3 * k + 2] = t.z;
        for (int i = 0; i < 4; i++)
            for (int j = 0; j < 3; j++) nn[12 * k + 3 * i + j] = t.nn[i][j];
        kind[k] = kd;
        evc[k] = t.ev;
        rate[k] = t.rate;
    }
    return 0;
}

int observables(State *s, mks_observables *o, std::string &err)
{
    memset(o, 0, sizeof *o);
    int top = 0;
    SK(cudaMemcpyAsync(&top, s->D.top, sizeof top, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaStreamSynchronize(s->stream));
    const int ncol = (s->D.lx / 6) * (s->D.ly / 6);
    unsigned long long *d_cnt = nullptr;
    double *d_rs = nullptr;
    int32_t *d_col = nullptr;
    SK(cudaMallocAsync(&d_cnt, sizeof(unsigned long long) * 8, s->stream));
    SK(cudaMallocAsync(&d_rs, sizeof(double) * 2, s->stream));
    SK(cudaMallocAsync(&d_col, sizeof(int32_t) * ncol, s->stream));
    SK(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long) * 8, s->stream));
    SK(cudaMemsetAsync(d_rs, 0, sizeof(double) * 2, s->stream));
    SK(cudaMemsetAsync(d_col, 0xff, sizeof(int32_t) * ncol, s->stream));
    if (top > 1) k_observe<<<grid_for(top), 256, 0, s->stream>>>(s->D, top, d_cnt, d_rs, d_col);
    SK(cudaGetLastError());
    unsigned long long cnt[8];
    double rs[2];
    std::vector<int32_t> col(ncol);
    SK(cudaMemcpyAsync(cnt, d_cnt, sizeof cnt, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaMemcpyAsync(rs, d_rs, sizeof rs, cudaMemcpyDeviceToHost, s->stream));
    SK(cudaMemcpyAsync(col.data(), d_col, sizeof(int32_t) * ncol, cudaMemcpyDeviceToHost, s->stream));
    cudaFreeAsync(d_cnt, s->stream);
    cudaFreeAsync(d_rs, s->stream);
    cudaFreeAsync(d_col, s->stream);
    SK(cudaStreamSynchronize(s->stream));
    o->events = s->events;
    o->time = s->time;
    o->atoms = (int64_t)cnt[0];
    o->undercoord = (int64_t)cnt[1];
    o->mc_sites = (int64_t)cnt[2];
    o->voids = (int64_t)cnt[3];
    for (int k = 0; k < 3; k++) o->species[k] = (int64_t)cnt[4 + k];
    o->nonepitaxial = (int64_t)cnt[7];
    o->total_rate = rs[0] + rs[1] * 1.0e5 * rs[0];
    double sh = 0.0, sh2 = 0.0;
    int64_t m = 0;
    for (int32_t h : col)
        if (h >= 0) {
            sh += h;
            sh2 += (double)h * h;
            m++;
        }
    if (m) {
        o->mean_height = sh / (double)m;
        double var = sh2 / (double)m - o->mean_height * o->mean_height;
        o->rms_roughness = sqrt(var > 0.0 ? var : 0.0);
    }
    return 0;
}

int clock(State *s, double *time, int64_t *window, int64_t *events)
{
    if (time) *time = s->time;
    if (window) *window = s->window;
    if (events) *events = s->events;
    return 0;
}

int status(State *s, mks_status *st)
{
    memset(st, 0, sizeof *st);
    st->error = s->last_error;
    st->windows = s->window;
    st->active = s->stop_reason == 0;
    st->stop_reason = s->stop_reason;
    return 0;
}

}  // namespace mks_stk
