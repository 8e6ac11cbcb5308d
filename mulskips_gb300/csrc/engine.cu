// engine.cu — GB300 (sm_103a) synchronous-sublattice KMC engine for the
// MulSKIPS event loop, and the C ABI declared in include/mulskips_gpu.h.
//
// Data layout in HBM (per replica): one byte per diamond site (lattice.cuh),
// layer-major st[z1][b][a] with rows padded to 16 bytes.  Each replica's
// (a,b) plane is cut into an even number of tiles per side; the four tile
// colours (tile index parity in a and b) form the four sublattices of the
// synchronous-sublattice method (Shim & Amar, Phys. Rev. B 71, 125432).  In
// one window of length tau every colour in turn advances all of its tiles
// from T0 to T0+tau; tiles of one colour are two tiles apart, so their event
// neighbourhoods (read range two bonds = 2 columns, write range one bond)
// never meet.  One warp runs one tile: it stages the tile plus a two-column
// halo and the surface band of layers in shared memory, builds the tile's
// list of event sites with per-class counts (warp ballot / popc), and then
// selects events rejection-free: class by cumulative rate (warp scan), member
// by a ballot scan of the class.  Rates are an FP32 table per class; the tile
// clock is FP64.  The reference's serial loop is mulskips-source/main.f:304-371.
#include <cuda.h>            // CUtensorMap and its enums (the encoder is fetched at run time)
#include <nvtx3/nvToolsExt.h>  // named ranges for profiler timelines (header-only)
#include <cuda_runtime.h>
#include <stdint.h>
#include <stdio.h>
#include <stdarg.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <string>
#include <vector>
#include <algorithm>
#include <unordered_map>

#include "lattice.cuh"
#include "shapes.cuh"
#include "tiling.cuh"
#include "rng.cuh"
#include "stacking.cuh"
#include "sicsf.h"
#include "../../include/mulskips_gpu.h"

using namespace mks;

namespace {

// ---------------------------------------------------------------- limits
constexpr int QMAX = mks_tiling::QMAX;   // max tile width (sites) in a or b
constexpr int HALO = 2;                  // read range of an event, in columns
constexpr int WB_MAX = QMAX + 2 * HALO;  // 12: staged rows per layer
constexpr int RS = 32;                   // staged row stride: one aligned 32-byte row segment
constexpr int WMAX = 20;                 // max staged layers
constexpr int MCCAP = 512;               // max event sites per tile
constexpr int ZMARGIN = 2;               // extra staged layers beyond the band on each side
constexpr int NRELOAD = 512;             // bounded re-staging per tile and phase

// device error codes (status word)
constexpr int DERR_INVARIANT = MKS_ERR_INVARIANT;
constexpr int DERR_CAPACITY = MKS_ERR_CAPACITY;
constexpr int DERR_TIMEOUT = MKS_ERR_TIMEOUT;

struct RepDev {
    int64_t st_off;
    int NA, NB, NZ, pitch;
    int nqa, nqb, quad_base;
    int single;              // NCrystal = 1: only species 1 on the lattice
    int cov;                 // coverage species (0..2): species value 3 is a covered empty site, bit 7 which
    double tau, T0, t_max;
    long long ev_max;
    unsigned long long seed;
    unsigned long long events;
    long long mc_count;
    unsigned int window;
    int active, stop_reason;
    int qshift;              // brick tiling: columns by which the tiles of odd rows are shifted (0: square grid)
    float rate[64];          // per class; CLS_ISO is computed per event
    float spcum[3][4];       // per coordination: cumulative fractions of species 1, 1+2, all deposition,
                             // deposition + absorption of coverage species 1
};

struct QuadDev {
    int rep, a0, a1, b0, b1;
    int zlo, zhi, mc;        // mutable: band of event sites and their count
    int qa, qb, colour;
    int ncol;                // colours of the replica's tiling: 4 square grid, 3 brick
    int ev;                  // events of this tile since the last window end (k_window_end folds them)
    int nbr[8];              // the eight neighbouring tiles (periodic)
};

// Laser-anneal rate law of the reference (mulskips-source/mcevent/Get_Prob.f:
// 127-149): the PTransE / PTransD tables hold barriers in eV and the rates
// follow the site temperature.  Melting of an atom of class c:
//   P0(s) exp(-E_c / kB T); solidification of species s on a liquid (empty)
// site of coordination n: 0.5 P0(s) exp(-Ed(s,n) / kB Tm(s)) (1 + erf((T -
// Tflex(s)) / sigma(s))); a zero barrier means no such event.  The
// temperature is the prescribed field T(z,t) = Tb + Ta exp(-((t-t0)/w)^2)
// exp(-depth/L), depth = max(0, (zsurf - z) sf / 10) nm, rounded to integer K
// as LattCoo bits 9-21 store it, evaluated at the window's midpoint.
constexpr int LA_NTAB = 32;                  // temperatures of a tabulated rate law

struct LADev {
    // crystal atoms per species: init_cnt at mks_batch_set_la, cnt updated by
    // the tiles (atomics); the liquid of species s is init_cnt[s] - cnt[s]
    // (CountLiquid = InitCountCrystal - CountCrystal, LaserAnnealing
    // main.f:637) and xliq its fraction, refreshed every LA_PHASE windows
    long long init_cnt[3];
    long long cnt[3];
    float xliq[3];
    int on, score_on;
    int swap_species;        // SiGe (14, 32) with liquid fractions: the species swap of LaserAnnealing main.f:676-681
    float P0[3], Tm[3], Tflex[3], sigma[3];
    float E[64];             // melting barrier of each occupied class
    float dE[64][4];         // d E / d theta
    float Edep[3][3];        // solidification barrier [species][coordination-1]
    float dEdep[3][3][4];
    float Tb, Ta, t0, w;
    float L, zsurf, sf;
    int liquid_weighting;    // 0: the MS law (no liquid fraction, no vacuum, no stop rule)
    // optional static per-site temperature (K, the LattCoo T bits of SetT),
    // same layout as the lattice, and its maximum per layer
    const uint16_t *tfield;
    const float *tlayer;
    int tNA, tNB, tpitch;
    // tabulated rates instead of the law above (InitSt ST, SetProbabilityFromField.f,
    // InterpProbFromField.f): class rates and deposition rates at ntab
    // temperatures, linear in T between them (0: not tabulated)
    int ntab;
    float tabT[LA_NTAB];
    float tabE[LA_NTAB][64];
    float tabD[LA_NTAB][3][3];
};

constexpr float KB_EV_F = 8.617330350e-5f;   // Get_Prob.f:70
constexpr int LA_PHASE = 8;                  // windows between liquid-fraction refreshes

__device__ __forceinline__ float la_temp(const LADev &A, int z1, double t)
{
    float depth = fmaxf(0.f, (A.zsurf - 3.f * (float)z1) * A.sf * 0.1f);
    float g = (float)((t - (double)A.t0) / (double)A.w);
    return rintf(A.Tb + A.Ta * __expf(-g * g) * __expf(-depth / A.L));
}
// temperature of site (a, b, z1): the static field when one is loaded, else
// the prescribed T(z, t)
__device__ __forceinline__ float la_temp_at(const LADev &A, int a, int b, int z1, double t)
{
    // a tile of a shifted brick row runs over the periodic edge: a may be >= NA
    if (A.tfield) return (float)__ldg(&A.tfield[((int64_t)z1 * A.tNB + b) * A.tpitch + (a >= A.tNA ? a - A.tNA : a)]);
    return la_temp(A, z1, t);
}
// row i and upper weight w of temperature T in the table: T between tabT[i]
// and tabT[i+1] (clamped to the table's ends)
__device__ __forceinline__ void la_tab_at(const LADev &A, float T, int &i, float &w)
{
    i = 0;
    w = 0.f;
    if (T <= A.tabT[0]) return;
    if (T >= A.tabT[A.ntab - 1]) {
        i = A.ntab - 1;
        return;
    }
    while (i + 2 < A.ntab && A.tabT[i + 1] <= T) i++;
    w = (T - A.tabT[i]) / (A.tabT[i + 1] - A.tabT[i]);
}
__device__ __forceinline__ float la_tab_mix(const LADev &A, int i, float w, float lo, float hi)
{
    return w > 0.f ? (1.f - w) * lo + w * hi : lo;
}
__device__ __forceinline__ float la_dep(const LADev &A, int s, int co, float T)
{
    if (A.ntab) {
        int i;
        float w;
        la_tab_at(A, T, i, w);
        return la_tab_mix(A, i, w, A.tabD[i][s][co - 1], w > 0.f ? A.tabD[i + 1][s][co - 1] : 0.f);
    }
    // LaserAnnealing Get_Prob.f:147-151: weighted by the liquid fraction of s
    float E = A.Edep[s][co - 1];
    if (E == 0.f || !(A.xliq[s] > 0.f)) return 0.f;
    return 0.5f * A.P0[s] * A.xliq[s] * __expf(-E / (KB_EV_F * A.Tm[s])) *
           (1.f + erff((T - A.Tflex[s]) / A.sigma[s]));
}
__device__ __forceinline__ int la_coor(int c) { return c == CLS_C3 ? 3 : (c == CLS_C2 ? 2 : 1); }
// rate of one site of class c at temperature T
__device__ __forceinline__ float la_rate(const LADev &A, int c, float T)
{
    if (A.ntab && c >= CLS_OCC0 && c < CLS_C1I) {
        int i;
        float w;
        la_tab_at(A, T, i, w);
        return la_tab_mix(A, i, w, A.tabE[i][c], w > 0.f ? A.tabE[i + 1][c] : 0.f);
    }
    if (c >= CLS_OCC0 && c < CLS_C1I) {
        float E = A.E[c];
        return E != 0.f ? A.P0[(c - CLS_OCC0) / NCENSUS] * __expf(-E / (KB_EV_F * T)) : 0.f;
    }
    if (c == CLS_C1 || c == CLS_C2 || c == CLS_C3) {
        int co = la_coor(c);
        return la_dep(A, 0, co, T) + la_dep(A, 1, co, T) + la_dep(A, 2, co, T);
    }
    if (c == CLS_C1D) return 1.e-8f;     // Get_Prob.f:183
    if (c == CLS_C1I) return 1.e-6f;     // Get_Prob_Ini.f:104
    return 0.f;
}
// Empty sites above the initial surface are vacuum, not liquid: nothing
// solidifies there (the liquid of the reference's LA runs is the molten part
// of the initially occupied domain, LaserAnnealing main.f:597-637)
__device__ __forceinline__ bool la_vacuum(const LADev &A, int c, int z1)
{
    return A.liquid_weighting && (c == CLS_C1 || c == CLS_C2 || c == CLS_C3) && 3.f * (float)z1 > A.zsurf;
}
// d(rate)/d theta_j of one site of class c at temperature T (isolated atoms,
// whose rate is a numerical device of the reference, are left out)
__device__ __forceinline__ void la_drate(const LADev &A, int c, float T, float d[4], bool vac = false)
{
    d[0] = d[1] = d[2] = d[3] = 0.f;
    if (vac) return;
    if (c >= CLS_OCC0 && c < CLS_C1I) {
        float k = la_rate(A, c, T);
        for (int j = 0; j < 4; j++) d[j] = -k * A.dE[c][j] / (KB_EV_F * T);
    } else if (c == CLS_C1 || c == CLS_C2 || c == CLS_C3) {
        int co = la_coor(c);
        for (int s = 0; s < 3; s++) {
            float k = la_dep(A, s, co, T);
            if (k == 0.f) continue;
            for (int j = 0; j < 4; j++) d[j] -= k * A.dEdep[s][co - 1][j] / (KB_EV_F * A.Tm[s]);
        }
    }
}

struct DevStatus {
    int error;               // first error code; nonzero also tells waiting warps to leave
    int err_quad;
    unsigned long long fallback;
    unsigned long long reloads;
};

__host__ __device__ __forceinline__ int wrapi(int v, int n) { return v < 0 ? v + n : (v >= n ? v - n : v); }

struct GLat {
    uint8_t *st;
    int NA, NB, NZ, pitch;
    // reads go to L2 (ld.global.cg): other SMs write the lattice during a
    // persistent launch and L1 is not coherent with them
    __device__ __forceinline__ uint8_t get(int a, int b, int z) const
    {
        if (z < 0 || z >= NZ) return 0;
        return __ldcg(&st[((int64_t)z * NB + wrapi(b, NB)) * pitch + wrapi(a, NA)]);
    }
    __device__ __forceinline__ void put(int a, int b, int z, uint8_t v) const
    {
        if (z < 0 || z >= NZ) return;
        st[((int64_t)z * NB + wrapi(b, NB)) * pitch + wrapi(a, NA)] = v;
    }
};

__device__ void set_error(DevStatus *s, int code, int quad)
{
    if (atomicCAS(&s->error, 0, code) == 0) s->err_quad = quad;
}

// --------------------------------------------------------------- kernels
// alloy_x > 0: substitutional species 2 on each occupied site with
// probability alloy_x (Philox on the site index, key alloy_seed), as SetSiGex
// places Ge at random (mulskips-source/initial/SetSiGex.f:60 uses RAND()).
__global__ void k_init_flat(uint8_t *st, int NA, int NB, int NZ, int pitch, int lz, int len1, int sic,
                            float alloy_x = 0.f, unsigned long long alloy_seed = 0ull)
{
    int64_t n = (int64_t)NZ * NB * pitch;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int a = (int)(i % pitch);
        int64_t r = i / pitch;
        int b = (int)(r % NB);
        int z = (int)(r / NB);
        uint8_t v = 0;
        if (a < NA && ((a + b + (z >> 1)) & 1) == 0) v = flat_init_state(z, lz, len1, sic != 0);
        if (alloy_x > 0.f && v != WALL && sp_of(v) == 1) {
            U4 r = philox4x32_10(U4{(uint32_t)i, (uint32_t)(i >> 32), 0x5147u, 0u}, (uint32_t)alloy_seed,
                                 (uint32_t)(alloy_seed >> 32));
            if (u01(r.x) < alloy_x) v = (uint8_t)((v & ~3) | 2);
        }
        st[i] = v;
    }
}

// Per-tile z range and count of event sites (and invariant check of the
// coordination bytes against the occupancy).
// Band scan of one replica: z band and count of the event sites of every
// tile.  One pass over the lattice in 16-byte units (thread per unit of a
// row), the site test from the byte alone, per-tile atomics for the few
// event sites.  k_band_init resets the replica's tiles first.
__global__ void k_band_init(QuadDev *quads, int q0, int nq)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < nq; i += gridDim.x * blockDim.x) {
        quads[q0 + i].zlo = 1 << 30;
        quads[q0 + i].zhi = -1;
        quads[q0 + i].mc = 0;
    }
}

__global__ void k_band_scan(const RepDev *reps, int rep, QuadDev *quads, const uint8_t *st_all, DevStatus *status)
{
    const RepDev &R = reps[rep];
    const uint4 *st = reinterpret_cast<const uint4 *>(st_all + R.st_off);
    const int upr = R.pitch / 16;
    const int64_t nu = (int64_t)R.NZ * R.NB * upr;
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nu; u += (int64_t)gridDim.x * blockDim.x) {
        uint4 v = __ldcs(st + u);
        if ((v.x | v.y | v.z | v.w) == 0u) continue;
        int64_t row = u / upr;
        int a0 = 16 * (int)(u - row * upr);
        int z = (int)(row / R.NB), b = (int)(row - (int64_t)z * R.NB);
        int qb = ((b + 1) * R.nqb - 1) / R.NB;       // the tile row holding b
        const uint8_t *by = reinterpret_cast<const uint8_t *>(&v);
        int q = -1, lo = 1 << 30, hi = -1, cnt = 0;
        bool bad = false;
#pragma unroll
        for (int k = 0; k < 16; k++) {
            int a = a0 + k;
            uint8_t sb = by[k];
            if (a >= R.NA || !event_byte(sb)) {
                if (R.single && sb != WALL && sp_of(sb) > 1) bad = true;
                continue;
            }
            if (R.single && sp_of(sb) > 1) bad = true;
            int qq = R.quad_base + mks_tiling::tile_of(R.NA, R.NB, R.nqa, R.nqb, R.qshift, a, b);
            if (qq != q) {
                if (q >= 0) {
                    atomicMin(&quads[q].zlo, lo);
                    atomicMax(&quads[q].zhi, hi);
                    atomicAdd(&quads[q].mc, cnt);
                }
                q = qq;
                lo = z;
                hi = z;
                cnt = 0;
            }
            cnt++;
        }
        if (q >= 0) {
            atomicMin(&quads[q].zlo, lo);
            atomicMax(&quads[q].zhi, hi);
            atomicAdd(&quads[q].mc, cnt);
        }
        if (bad) set_error(status, DERR_INVARIANT, R.quad_base + qb * R.nqa);   // species > 1 with NCrystal = 1
    }
}

// Class histograms from the tiles' z bands (which hold every event site):
// block per tile of replicas [rep0, rep1), hist[rep - rep0][class].
__global__ void k_class_hist(const RepDev *reps, const QuadDev *quads, int q0, int q1, int rep0, uint8_t *st_all,
                             unsigned long long *hist)
{
    __shared__ unsigned int sh[NCLASS];
    for (int q = q0 + blockIdx.x; q < q1; q += gridDim.x) {
        for (int i = threadIdx.x; i < NCLASS; i += blockDim.x) sh[i] = 0;
        __syncthreads();
        const QuadDev &Q = quads[q];
        const RepDev &R = reps[Q.rep];
        GLat L{st_all + R.st_off, R.NA, R.NB, R.NZ, R.pitch};
        int wa = Q.a1 - Q.a0, wb = Q.b1 - Q.b0;
        int zlo = max(0, Q.zlo), zhi = min(R.NZ - 1, Q.zhi);
        int n = (zhi - zlo + 1) * wa * wb;
        for (int i = threadIdx.x; i < n; i += blockDim.x) {
            int ia = i % wa, r = i / wa, ib = r % wb, z = zlo + r / wb;
            int a = Q.a0 + ia, b = Q.b0 + ib;
            if ((a + b + (z >> 1)) & 1) continue;
            if (!event_byte(L.get(a, b, z))) continue;
            atomicAdd(&sh[site_class(L, a, b, z, false, R.cov != 0, R.cov == 2)], 1u);
        }
        __syncthreads();
        for (int i = threadIdx.x; i < NCLASS; i += blockDim.x)
            if (sh[i]) atomicAdd(&hist[(size_t)(Q.rep - rep0) * NCLASS + i], (unsigned long long)sh[i]);
        __syncthreads();
    }
}

// Observables of one replica, pass 1: thread per (64-layer slab, row b,
// 16-column unit) with 16-byte loads; counts reduced per warp, the top atom of
// each column within the slab stored in top[(slab * NB + b) * NA + a] (-1:
// none).
constexpr int OBS_ZSLAB = 64;
__global__ void k_observables(const RepDev *reps, int rep, uint8_t *st_all, unsigned long long *cnt, int *top)
{
    const RepDev &R = reps[rep];
    const uint8_t *st = st_all + R.st_off;
    const int upr = R.pitch / 16, nslab = (R.NZ + OBS_ZSLAB - 1) / OBS_ZSLAB;
    const int64_t zs = (int64_t)R.NB * R.pitch;
    const bool covm = R.cov != 0;
    unsigned long long atoms = 0, under = 0, voids = 0, sp1 = 0, sp2 = 0, sp3 = 0;
    for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < (int64_t)nslab * R.NB * upr;
         t += (int64_t)gridDim.x * blockDim.x) {
        int unit = (int)(t % upr);
        int64_t r = t / upr;
        int b = (int)(r % R.NB), slab = (int)(r / R.NB);
        int a0 = 16 * unit, z0 = slab * OBS_ZSLAB, z1 = min(R.NZ, z0 + OBS_ZSLAB);
        int tk[16];
#pragma unroll
        for (int k = 0; k < 16; k++) tk[k] = -1;
        const uint8_t *col = st + (int64_t)b * R.pitch + a0;
        for (int zb = z0; zb < z1; zb += 4) {
            uint4 v[4];
#pragma unroll
            for (int u = 0; u < 4; u++)
                if (zb + u < z1) v[u] = __ldcs(reinterpret_cast<const uint4 *>(col + (zb + u) * zs));
#pragma unroll
            for (int u = 0; u < 4; u++) {
                int z = zb + u;
                if (z >= z1) break;
                if ((v[u].x | v[u].y | v[u].z | v[u].w) == 0u) continue;
                const uint8_t *by = reinterpret_cast<const uint8_t *>(&v[u]);
                int par = (a0 + b + (z >> 1)) & 1;     // a0 is even: byte k is a site iff k+par even
#pragma unroll
                for (int k = 0; k < 16; k++) {
                    uint8_t sb = by[k];
                    if (((k + par) & 1) || sb == 0 || sb == WALL) continue;
                    int sp = sp_of(sb), co = co_of(sb);
                    if (covm && sp == COVSP) {         // covered empty site: counted in the species-3 slot
                        sp3++;
                        voids += co == 4;
                    } else if (sp) {
                        atoms++;
                        under += co <= 3;
                        sp1 += sp == 1;
                        sp2 += sp == 2;
                        sp3 += sp == 3;
                        tk[k] = z;
                    } else {
                        voids += co == 4;
                    }
                }
            }
        }
        int *tp = top + ((int64_t)slab * R.NB + b) * R.NA + a0;
#pragma unroll
        for (int k = 0; k < 16; k++)
            if (a0 + k < R.NA) tp[k] = tk[k];
    }
    unsigned long long c[6] = {atoms, under, voids, sp1, sp2, sp3};
#pragma unroll
    for (int j = 0; j < 6; j++) {
        unsigned long long x = c[j];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(&cnt[j], x);
    }
}

// Atoms per species of every replica in one launch: grid (x blocks, replicas),
// 16-byte units, counts reduced per warp into cnt[3 * rep + species - 1].
__global__ void k_species_counts(const RepDev *reps, int rep0, const uint8_t *st_all, unsigned long long *cnt)
{
    const int rep = rep0 + (int)blockIdx.y;
    const RepDev &R = reps[rep];
    const uint4 *st = reinterpret_cast<const uint4 *>(st_all + R.st_off);
    const int64_t nu = (int64_t)R.NZ * R.NB * (R.pitch / 16);
    unsigned long long c[3] = {0, 0, 0};
    for (int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; u < nu; u += (int64_t)gridDim.x * blockDim.x) {
        uint4 v = __ldcs(st + u);
        if ((v.x | v.y | v.z | v.w) == 0u) continue;
        const uint8_t *by = reinterpret_cast<const uint8_t *>(&v);
#pragma unroll
        for (int k = 0; k < 16; k++) {
            uint8_t sb = by[k];
            int sp = sp_of(sb);
            if (sb == WALL || !sp) continue;
            c[0] += sp == 1;
            c[1] += sp == 2;
            c[2] += sp == 3;
        }
    }
#pragma unroll
    for (int j = 0; j < 3; j++) {
        unsigned long long x = c[j];
        for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
        if ((threadIdx.x & 31) == 0 && x) atomicAdd(&cnt[3 * rep + j], x);
    }
}

// pass 2: per column the highest slab top; mean and mean square of the
// column heights (top atom, grid units)
__global__ void k_observables_heights(const int *top, int64_t ncol, int nslab, unsigned long long *cnt, double *hsum)
{
    double h1 = 0.0, h2 = 0.0;
    unsigned long long cols = 0;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < ncol; i += (int64_t)gridDim.x * blockDim.x) {
        int tz = -1;
        for (int sl = nslab - 1; sl >= 0 && tz < 0; sl--) tz = top[(int64_t)sl * ncol + i];
        if (tz < 0) continue;
        double hh = 3.0 * tz;
        h1 += hh;
        h2 += hh * hh;
        cols++;
    }
    for (int o = 16; o > 0; o >>= 1) {
        h1 += __shfl_xor_sync(0xffffffffu, h1, o);
        h2 += __shfl_xor_sync(0xffffffffu, h2, o);
        cols += __shfl_xor_sync(0xffffffffu, cols, o);
    }
    if ((threadIdx.x & 31) == 0 && cols) {
        atomicAdd(&hsum[0], h1);
        atomicAdd(&hsum[1], h2);
        atomicAdd(&cnt[6], cols);
    }
}

// Rate class and rate of given sites (grid coordinates, as AtomXYZ of the
// reference's ListAdAtom): the ProbTrans the reference keeps in its tree
// leaves (Get_Prob / Get_Prob_Ini).  Isolated atoms get rate 0 here (their
// rate, 1e5 x Tree(1), follows the total); LA replicas take the rate law at
// the site's temperature at the replica's clock.  A grid point that is not a
// diamond site of the box gets class -1.
__global__ void k_site_rates(const RepDev *reps, int rep, const uint8_t *st_all, const LADev *la, const int32_t *xyz,
                             int64_t n, int32_t *cls, float *rate)
{
    const RepDev &R = reps[rep];
    GLat L{const_cast<uint8_t *>(st_all) + R.st_off, R.NA, R.NB, R.NZ, R.pitch};
    const LADev *A = (la && la[rep].on) ? &la[rep] : nullptr;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int x = xyz[3 * i], y = xyz[3 * i + 1], z = xyz[3 * i + 2];
        int x1 = x / 3, y1 = y / 3, z1 = z / 3, a = x1 >> 1, b = y1 >> 1;
        bool ok = x >= 0 && y >= 0 && z >= 0 && x % 3 == 0 && y % 3 == 0 && z % 3 == 0 && ((x1 & 1) == (z1 & 1)) &&
                  ((y1 & 1) == (z1 & 1)) && z1 < R.NZ && a < R.NA && b < R.NB && ((a + b + (z1 >> 1)) & 1) == 0;
        if (!ok) {
            cls[i] = -1;
            rate[i] = 0.f;
            continue;
        }
        int c = site_class(L, a, b, z1, R.single != 0, R.cov != 0, R.cov == 2);
        float r = 0.f;
        if (c != CLS_ISO && c != CLS_NONE)
            r = A ? la_rate(*A, c, la_temp_at(*A, a, b, z1, R.T0)) : R.rate[c];
        cls[i] = c;
        rate[i] = r;
    }
}

// Apply a given event sequence in order (one thread; the sequence is serial by
// definition).  Deposition.f / Evaporation.f restated in lattice.cuh.
__global__ void k_replay(const RepDev *reps, uint8_t *st_all, const mks_event *ev, int64_t n, DevStatus *status,
                         long long *done)
{
    if (threadIdx.x != 0 || blockIdx.x != 0) return;
    const RepDev &R = reps[0];
    GLat L{st_all + R.st_off, R.NA, R.NB, R.NZ, R.pitch};
    for (int64_t i = 0; i < n; i++) {
        mks_event e = ev[i];
        int x1 = e.x / 3, y1 = e.y / 3, z1 = e.z / 3;
        int a = x1 >> 1, b = y1 >> 1;
        bool ok = (e.x % 3 == 0) && (e.y % 3 == 0) && (e.z % 3 == 0) && ((x1 & 1) == (z1 & 1)) &&
                  ((y1 & 1) == (z1 & 1)) && e.x >= 0 && e.y >= 0 && z1 >= 0 && z1 < R.NZ && a < R.NA &&
                  b < R.NB && e.arm == 0;
        const bool cov = R.cov != 0;
        int c = ok ? site_class(L, a, b, z1, false, cov, R.cov == 2) : CLS_NONE;
        bool atom_cls = c == CLS_ISO || ((cov ? c >= CLS_COV0 : c >= CLS_OCC0) && c < CLS_C1I);
        Touched tc;
        int err = 1;
        if (ok && c != CLS_NONE) {
            if (e.itrans >= 1 && e.itrans <= 3 && dep_class(c))
                err = apply_deposition(L, a, b, z1, e.itrans, tc, cov);
            else if (e.itrans == 4 && atom_cls)
                err = apply_evaporation(L, a, b, z1, tc, cov);
            else if (cov && e.itrans == 5 &&
                     ((c >= CLS_D1 && c < CLS_COV0) || (R.cov == 2 && c >= CLS_D2 && c < CLS_D2 + 3)))
                err = apply_coverage(L, a, b, z1, false, tc);    // desorption, main.f:346-349
            else if (cov && e.itrans >= 6 && e.itrans - 5 <= R.cov && c >= CLS_C1 && c <= CLS_C3 && c != CLS_C1D)
                err = apply_coverage(L, a, b, z1, true, tc, e.itrans - 5);   // absorption of ListCov(Itrans-5), :350-356
        }
        if (err) {
            set_error(status, DERR_INVARIANT, (int)i);
            *done = i;
            return;
        }
    }
    *done = n;
}

// ------------------------------------------------ the sublattice kernel
struct __align__(128) TileShared {
    uint8_t win[RS * WB_MAX * WMAX];           // staged rows, 32-byte aligned segments (TMA box target)
    uint32_t list[MCCAP];                      // (site key << 8) | class; class 0 = dead entry
    uint16_t pos[QMAX * QMAX * WMAX];          // list slot of each listed tile site (others stale: checked against list)
    int cnt[64];
    float rate[64];
    float spcum[3][4];
    float G[4];                                // LA: sum over event sites of d(rate)/d(theta)
    int dcnt[3];                               // LA: net crystal atoms per species added by this tile
    int nlist;
    int rate_rep;                              // replica whose rate table is in rate/spcum (-1 none)
    unsigned long long mbar;                   // TMA staging barrier
    unsigned int tma_phase;                    // its parity
    // persistent schedule, a colour with exactly one tile of this warp: the
    // tile's colour count (0 otherwise) and, per neighbour k, (tile << 2) |
    // phase lag -- fixed for the launch, so the flag polls start without
    // global reads
    int one_ncol[4];
    int one_nb[4][8];
};

// The one tile a warp works on (one warp per block).  Declared at file scope so
// every access compiles to shared-memory instructions.
__shared__ TileShared g_tile;

// ---- TMA staging: one cp.async.bulk.tensor per 4 layers of the band ----
// tensor map per replica: dims (pitch, NB, NZ) bytes, box (32, WB_MAX, 4)
constexpr int TMA_BZ = 4;
constexpr unsigned TMA_BOX_BYTES = RS * WB_MAX * TMA_BZ;
constexpr long long TMA_WAIT_LIMIT = 1LL << 22;      // try_wait polls before the copy is declared lost
static_assert(WMAX % TMA_BZ == 0, "staged layers must be whole boxes");

__device__ __forceinline__ uint32_t smem_addr(const void *p) { return (uint32_t)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void tma_barrier_init()
{
    if ((threadIdx.x & 31) == 0) {
        asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(smem_addr(&g_tile.mbar)) : "memory");
        asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
        g_tile.tma_phase = 0;
    }
    __syncwarp();
}

// Stage layers [zw0, zw0 + wz) of the rows bx0.. (WB_MAX of them) and the 32
// columns from ax0 (a multiple of 16) into g_tile.win.  Returns false if the
// copy did not complete within the wait limit.
__device__ __forceinline__ bool tma_stage(const CUtensorMap *tmap, int ax0, int bx0, int zw0, int wz)
{
    int lane = threadIdx.x & 31;
    uint32_t mb = smem_addr(&g_tile.mbar);
    uint32_t ph = g_tile.tma_phase;
    int nbox = (wz + TMA_BZ - 1) / TMA_BZ;
    __syncwarp();
    if (lane == 0) {
        // earlier generic accesses (this warp's shared reads/writes, the
        // neighbours' global writes it acquired) before the async copies
        asm volatile("fence.proxy.async;" ::: "memory");
        asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mb), "r"(nbox * TMA_BOX_BYTES)
                     : "memory");
        for (int i = 0; i < nbox; i++)
            asm volatile(
                "cp.async.bulk.tensor.3d.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3, %4}], "
                "[%5];" ::"r"(smem_addr(&g_tile.win[i * TMA_BZ * WB_MAX * RS])),
                "l"(reinterpret_cast<uint64_t>(tmap)), "r"(ax0), "r"(bx0), "r"(zw0 + i * TMA_BZ), "r"(mb)
                : "memory");
    }
    uint32_t done = 0;
    for (long long it = 0; it < TMA_WAIT_LIMIT && !done; it++)
        asm volatile("{ .reg .pred p; mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2; selp.u32 %0, 1, 0, p; }"
                     : "=r"(done)
                     : "r"(mb), "r"(ph)
                     : "memory");
    bool ok = __all_sync(0xffffffffu, done != 0);
    if (lane == 0) g_tile.tma_phase = ph ^ 1u;
    __syncwarp();
    return ok;
}

// Staged window with write-through: every byte an event writes goes to the
// shared copy and, at once, to the lattice in global memory, so the stores
// drain while the tile keeps working and the phase ends without a write-back
// pass.  No other tile reads or writes these bytes during the phase (same-
// colour tiles are two tiles apart; the others wait for this tile's flag).
struct SLat {
    int ax0, bx0, zw0, NZ;   // (a, b, z) of staged byte 0
    uint8_t *st;             // the replica's lattice
    int NA, NB, pitch;
    __device__ __forceinline__ uint8_t get(int a, int b, int z) const
    {
        if (z < 0 || z >= NZ) return 0;
        return g_tile.win[((z - zw0) * WB_MAX + (b - bx0)) * RS + (a - ax0)];
    }
    __device__ __forceinline__ void put(int a, int b, int z, uint8_t v) const
    {
        if (z < 0 || z >= NZ) return;
        g_tile.win[((z - zw0) * WB_MAX + (b - bx0)) * RS + (a - ax0)] = v;
        st[((int64_t)z * NB + wrapi(b, NB)) * pitch + wrapi(a, NA)] = v;
    }
};

// Replica scalars the tile kernels need, held in registers.
struct RepLocal {
    int64_t st_off;
    int NA, NB, NZ, pitch;
    double tau;
    unsigned long long seed;
    int active, single, cov;
};
__device__ __forceinline__ RepLocal rep_local(const RepDev &R)
{
    RepLocal r;
    r.st_off = R.st_off;
    r.NA = R.NA;
    r.NB = R.NB;
    r.NZ = R.NZ;
    r.pitch = R.pitch;
    r.tau = R.tau;
    r.seed = R.seed;
    r.active = R.active;
    r.single = R.single;
    r.cov = R.cov;
    return r;
}

__device__ __forceinline__ int key_of(int ia, int ib, int z) { return (z << 10) | (ib << 5) | ia; }
__device__ __forceinline__ int pos_index(uint32_t key, int zw0)
{
    return ((int)(key >> 10) - zw0) * (QMAX * QMAX) + (((int)(key >> 5) & 31) - HALO) * QMAX + ((int)(key & 31) - HALO);
}
__device__ __forceinline__ unsigned lanemask_lt() { return (1u << (threadIdx.x & 31)) - 1u; }

// Scan the tile's sites in layers [zl, zh] and build the event-site list and
// the class counts (ballot compaction, per-class counts aggregated with
// match_any).  pos covers the wz staged layers from zw0 (smem path only).
template <class Lat>
__device__ __forceinline__ bool build_list(const Lat &L, int a0, int b0, int wa, int wb, int zl, int zh,
                                           bool use_pos, int zw0, int wz, bool single, bool cov, bool cov2,
                                           const LADev *A = nullptr, double t_mid = 0.0)
{
    TileShared &S = g_tile;
    const unsigned FULL = 0xffffffffu;
    int lane = threadIdx.x & 31;
    // pos is not cleared: every listed site's slot is written below or on
    // append, and a lookup accepts a slot only if the list entry there holds
    // the same site key
    for (int c = lane; c < 64; c += 32) S.cnt[c] = 0;
    __syncwarp();
    // lanes walk the diamond sites of the band only: per layer, row ib holds
    // the sites ia = 2 ja + p with p the row's parity, ja < ceil(wa/2)
    const int hw = (wa + 1) >> 1, per = wb * hw, nsl = per * (zh - zl + 1);
    int nl = 0;
    float g[4] = {0.f, 0.f, 0.f, 0.f};
    // site s0 + lane is (layer dz, index k) with k = ib * hw + ja; both are
    // advanced by 32 sites per step without divisions (k / hw by a 16-bit
    // reciprocal: exact for k < 64 and hw <= 4)
    int dz = lane / per, k = lane - dz * per;
    const unsigned hmul = 65536u / (unsigned)hw + 1u;
    for (int s0 = 0; s0 < nsl; s0 += 32) {
        int sidx = s0 + lane;
        int cls = CLS_NONE, ia = 0, ib = 0, z = zl;
        if (sidx < nsl) {
            z = zl + dz;
            ib = (int)(((unsigned)k * hmul) >> 16);
            ia = 2 * (k - ib * hw) + ((a0 + b0 + ib + (z >> 1)) & 1);
            if (ia < wa) cls = site_class(L, a0 + ia, b0 + ib, z, single, cov, cov2);
        }
        k += 32;
        while (k >= per) {
            k -= per;
            dz++;
        }
        unsigned m = __ballot_sync(FULL, cls != CLS_NONE);
        if (cls != CLS_NONE) {
            uint32_t key = (uint32_t)key_of(ia + HALO, ib + HALO, z);
            int slot = nl + __popc(m & lanemask_lt());
            if (slot < MCCAP) {
                S.list[slot] = (key << 8) | (uint32_t)cls;
                if (use_pos) S.pos[pos_index(key, zw0)] = (uint16_t)slot;
            }
            atomicAdd(&S.cnt[cls], 1);
            if (A) {
                float d[4];
                la_drate(*A, cls, la_temp_at(*A, a0 + ia, b0 + ib, z, t_mid), d, la_vacuum(*A, cls, z));
                for (int j = 0; j < 4; j++) g[j] += d[j];
            }
        }
        nl += __popc(m);
    }
    if (A) {
        for (int j = 0; j < 4; j++) {
            float v = g[j];
            for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
            if (lane == 0) S.G[j] = v;
        }
    }
    if (lane == 0) S.nlist = min(nl, MCCAP);
    __syncwarp();
    return nl <= MCCAP;
}

// Run events of one tile on accessor L until the tile clock reaches t_end,
// the tile has no events, or an event would read outside the staged layers.
// Returns 0 done, 1 needs re-staging, <0 error.  hz_lo/hz_hi (per lane) collect
// the layers of changed sites outside the tile.
template <class Lat>
__device__ __forceinline__ int run_events(Lat &L, const RepLocal &R, const QuadDev &Q, int qid, double &t,
                                          double t_end, unsigned int &evc, int zw0, int zw1, bool use_pos,
                                          int &hz_lo, int &hz_hi, unsigned long long &nev, uint32_t k0, uint32_t k1,
                                          uint32_t phase_tag, unsigned int window, const LADev *A = nullptr,
                                          double t_mid = 0.0, double *sc = nullptr)
{
    TileShared &S = g_tile;
    // LA score: G (uniform over lanes) and the accumulator sc (lane 0, FP64)
    float G[4] = {0.f, 0.f, 0.f, 0.f};
    if (A && sc)
        for (int j = 0; j < 4; j++) G[j] = S.G[j];
    const unsigned FULL = 0xffffffffu;
    int lane = threadIdx.x & 31;
    int wa = Q.a1 - Q.a0, wb = Q.b1 - Q.b0;
    const int NZ = R.NZ;
    // Philox draws of 32 consecutive events, one event per lane
    unsigned int pre_base = evc;
    U4 pre = philox4x32_10(U4{pre_base + (unsigned)lane, (uint32_t)qid, window, phase_tag}, k0, k1);
    int used = 0;
    bool fresh = true;                                 // no event since the list was built
    // time left in the window, FP32 on the critical path; the FP64 clock t is
    // still accumulated event by event
    float rem = (float)(t_end - t);
    // lane l owns classes 2l and 2l+1 (ISO apart); the class rates stay fixed
    // while the tile runs
    const int c0 = 2 * lane, c1 = 2 * lane + 1;
    const float rate0 = (c0 < NCLASS && c0 != CLS_ISO) ? S.rate[c0] : 0.f;
    const float rate1 = (c1 < NCLASS && c1 != CLS_ISO) ? S.rate[c1] : 0.f;
    for (;;) {
        int nlist = S.nlist;
        if (nlist > MCCAP - 5) return fresh ? -DERR_CAPACITY : 1;   // compact the list by re-staging
        // cumulative class weights
        float w0 = (float)S.cnt[c0] * rate0;
        float w1 = (float)S.cnt[c1] * rate1;
        float s = w0 + w1;
#pragma unroll
        for (int o = 1; o < 32; o <<= 1) {
            float v = __shfl_up_sync(FULL, s, o);
            if (lane >= o) s += v;
        }
        float r_rest = __shfl_sync(FULL, s, 31);
        int n_iso = S.cnt[CLS_ISO];
        float r_iso = n_iso ? (float)n_iso * 1.0e5f * fmaxf(r_rest, 1.0e-30f) : 0.f;
        float rtot = r_rest + r_iso;
        if (!(rtot > 0.f)) return 0;
        if (used == 32) {
            pre_base += 32;
            pre = philox4x32_10(U4{pre_base + (unsigned)lane, (uint32_t)qid, window, phase_tag}, k0, k1);
            used = 0;
        }
        U4 rnd;
        rnd.x = __shfl_sync(FULL, pre.x, used);
        rnd.y = __shfl_sync(FULL, pre.y, used);
        rnd.z = __shfl_sync(FULL, pre.z, used);
        rnd.w = __shfl_sync(FULL, pre.w, used);
        used++;
        evc++;
        float dt = __fdividef(-__logf(u01(rnd.z)), rtot);
        if (dt > rem) {
            if (sc && lane == 0)
                for (int j = 0; j < 4; j++) sc[j] -= (double)G[j] * (double)rem;
            t = t_end;
            return 0;
        }
        // class selection
        float target = u01(rnd.x) * rtot;
        int cls;
        if (target >= r_rest && n_iso > 0) {
            cls = CLS_ISO;
        } else {
            unsigned m = __ballot_sync(FULL, s > target);
            cls = -1;
            if (m) {
                int l = __ffs(m) - 1;
                float sl = __shfl_sync(FULL, s, l);
                float w0l = __shfl_sync(FULL, w0, l);
                float w1l = __shfl_sync(FULL, w1, l);
                float el = sl - w0l - w1l;
                cls = (target < el + w0l) ? 2 * l : 2 * l + 1;
                if (cls == 2 * l && !(w0l > 0.f)) cls = 2 * l + 1;
                if (cls == 2 * l + 1 && !(w1l > 0.f)) cls = (w0l > 0.f) ? 2 * l : -1;
            }
            if (cls < 0 || cls >= NCLASS || S.cnt[cls] == 0) {
                // rounding at the top end: take the last class with weight
                cls = -1;
                for (int c = NCLASS - 1; c >= 0; c--)
                    if (c != CLS_ISO && S.cnt[c] > 0 && S.rate[c] > 0.f) { cls = c; break; }
                if (cls < 0) return 0;
            }
        }
        // member selection: the k-th live list entry of class cls (ballot scan)
        int k = min((int)(u01(rnd.y) * (float)S.cnt[cls]), S.cnt[cls] - 1);
        int slot = -1;
        for (int base = 0; base < nlist; base += 32) {
            int i = base + lane;
            bool hit = i < nlist && (int)(S.list[i] & 0xFF) == cls;
            unsigned m = __ballot_sync(FULL, hit);
            int nh = __popc(m);
            if (k < nh) {
                // the lane holding the k-th hit of this chunk
                unsigned pick = __ballot_sync(FULL, hit && __popc(m & lanemask_lt()) == k);
                slot = base + __ffs(pick) - 1;
                break;
            }
            k -= nh;
        }
        if (slot < 0) return -DERR_INVARIANT;
        uint32_t key = S.list[slot] >> 8;
        int z = key >> 10;
        int a = Q.a0 + (int)(key & 31) - HALO, b = Q.b0 + (int)((key >> 5) & 31) - HALO;
        // every listed site lies inside the staged layers with its two-layer
        // read range (the list is built inside them and an event that lists a
        // site outside re-stages before the next draw, below), so a drawn event
        // is never set aside: throwing a draw away and drawing again would
        // under-sample the sites at the band's edges
        if ((z - 2 < zw0 && zw0 > 0) || (z + 3 > zw1 && zw1 < NZ)) return -DERR_INVARIANT;
        t += (double)dt;
        rem -= dt;
        if (sc && lane == 0)
            for (int j = 0; j < 4; j++) sc[j] -= (double)G[j] * (double)dt;
        int sp = 0;
        float Tsite = 0.f;
        if (A) {
            // thinning: the class rate is the tile's bound; accept with k(T_site)/bound
            Tsite = la_temp_at(*A, a, b, z, t_mid);
            if (cls != CLS_ISO) {
                float r_true = la_vacuum(*A, cls, z) ? 0.f : la_rate(*A, cls, Tsite);
                float uu = u01(rnd.y) * (float)S.cnt[cls];
                float uacc = uu - floorf(uu);
                if (!(uacc * S.rate[cls] < r_true)) continue;   // null event: time only
            }
        }
        int covev = 0;                                 // 1 absorption of ListCov(1), 2 desorption, 3 absorption of ListCov(2)
        if (R.cov && ((cls >= CLS_D1 && cls < CLS_COV0) || (R.cov == 2 && cls >= CLS_D2 && cls < CLS_D2 + 3))) {
            covev = 2;                                 // main.f:346-349
        } else if (dummy_class(cls)) {
            // unsupported coor-1 site: Get_Prob.f:181-184 (and Get_Prob_Ini.f:
            // 102-104) fix IndexEvent = 1 (species 1) with the dummy rate,
            // whatever the tables say
            sp = 1;
        } else if (cls >= CLS_C1 && cls <= CLS_C3) {
            int co = cls == CLS_C3 ? 3 : (cls == CLS_C2 ? 2 : 1);
            float u = u01(rnd.w);
            if (A) {
                float p1 = la_dep(*A, 0, co, Tsite), p2 = la_dep(*A, 1, co, Tsite), p3 = la_dep(*A, 2, co, Tsite);
                float tot = p1 + p2 + p3;
                sp = u * tot < p1 ? 1 : (u * tot < p1 + p2 ? 2 : 3);
                if (sc && lane == 0) {
                    int s0 = sp - 1;
                    for (int j = 0; j < 4; j++)
                        sc[j] += -(double)A->dEdep[s0][co - 1][j] / ((double)KB_EV_F * (double)A->Tm[s0]);
                }
                // LaserAnnealing main.f:676-681: SiGe solidification of a
                // species whose crystal count has reached its initial count
                // deposits the other one; the count is the replica's at the
                // last tile publication plus this tile's own changes (lane 0
                // reads it once, so every lane takes the same species)
                if (A->swap_species && sp <= 2) {
                    int sw = 0;
                    if (lane == 0)
                        sw = __ldcg(&A->cnt[sp - 1]) + (long long)S.dcnt[sp - 1] >= A->init_cnt[sp - 1] ? 1 : 0;
                    if (__shfl_sync(FULL, sw, 0)) sp = 3 - sp;
                }
            } else {
                sp = u < S.spcum[co - 1][0] ? 1 : (u < S.spcum[co - 1][1] ? 2 : 3);
                // past the deposition share: absorption of a coverage
                // species, the first up to its cumulative share
                // (Get_Prob.f:155-204, IndexEvent_Abs :22-52)
                if (R.cov && !(u < S.spcum[co - 1][2])) {
                    sp = 0;
                    covev = (R.cov == 2 && !(u < S.spcum[co - 1][3])) ? 3 : 1;
                }
            }
        } else if (A && sc && lane == 0 && cls >= CLS_OCC0 && cls < CLS_C1I) {
            for (int j = 0; j < 4; j++) sc[j] += -(double)A->dE[cls][j] / ((double)KB_EV_F * (double)Tsite);
        }
        int ta = a, tb = b, tz = z;
        if (covev) {
            // absorption.f / desorption.f: only the site byte changes; lanes
            // 1..4 take its neighbours for re-classification
            int v = lane == 0 ? cov_event_state(L, a, b, z, covev != 2, covev == 3 ? 2 : 1) : 0;
            if (__shfl_sync(FULL, v, 0) < 0) return -DERR_INVARIANT;
            __syncwarp();
            if (lane == 0) L.put(a, b, z, (uint8_t)v);
            if (lane >= 1 && lane <= 4) {
                int da, db, dz;
                nb_off(z & 1, lane - 1, da, db, dz);
                ta = a + da;
                tb = b + db;
                tz = z + dz;
            }
            __syncwarp();
        } else {
        // stage 1: the event site (every lane derives the context, lane 0 writes)
        EvCtx e;
        uint8_t sx0 = L.get(a, b, z);
        if (ev_prepare(sx0, a, b, z, sp, e, R.cov != 0)) return -DERR_INVARIANT;
        if (A && lane == 0) {
            if (sp) S.dcnt[sp - 1]++;
            else S.dcnt[sp_of(sx0) - 1]--;
        }
        if (lane == 0) L.put(a, b, z, ev_begin_state(e));
        __syncwarp();
        // stage 2: lanes 1..4 update the four neighbours, independent of one another
        int r2 = 0;
        if (lane >= 1 && lane <= 4) r2 = ev_neighbour(L, e, lane - 1, ta, tb, tz);
        unsigned wallm = __ballot_sync(FULL, lane >= 1 && lane <= 4 && r2 == 1);
        if (__ballot_sync(FULL, r2 < 0)) return -DERR_INVARIANT;
        __syncwarp();
        // stage 3: final state of the event site
        int r3 = 0;
        if (lane == 0) r3 = ev_finish(L, e, __popc(wallm));
        if (__shfl_sync(FULL, r3, 0)) return -DERR_INVARIANT;
        __syncwarp();
        }
        // re-classify the five touched sites, one per lane (lane 0 the event site)
        bool act = lane < 5 && tz >= 0 && tz < NZ;
        int ia = ta - Q.a0, ib = tb - Q.b0;
        bool interior = act && ia >= 0 && ia < wa && ib >= 0 && ib < wb;
        if (act && !interior) {
            hz_lo = min(hz_lo, tz);
            hz_hi = max(hz_hi, tz);
        }
        int ncls = interior ? site_class(L, ta, tb, tz, R.single != 0, R.cov != 0, R.cov == 2) : CLS_NONE;
        uint32_t tkey = interior ? (uint32_t)key_of(ia + HALO, ib + HALO, tz) : 0u;
        // old list slot of each touched site
        int my_slot = -1;
        if (use_pos) {
            if (interior) {
                int p = (int)S.pos[pos_index(tkey, zw0)];
                my_slot = (p < nlist && (S.list[p] >> 8) == tkey) ? p : -1;
            }
        } else {
            unsigned im = __ballot_sync(FULL, interior);
            while (im) {
                int src = __ffs(im) - 1;
                im &= im - 1;
                uint32_t kk = __shfl_sync(FULL, tkey, src);
                int found = -1;
                for (int base = 0; base < nlist && found < 0; base += 32) {
                    int i = base + lane;
                    unsigned m = __ballot_sync(FULL, i < nlist && (S.list[i] >> 8) == kk);
                    if (m) found = base + __ffs(m) - 1;
                }
                if (lane == src) my_slot = found;
            }
        }
        // update the list in one parallel step: entries leaving the list are
        // marked dead in place, new ones appended
        int old_cls = (interior && my_slot >= 0) ? (int)(S.list[my_slot] & 0xFF) : CLS_NONE;
        bool append = interior && my_slot < 0 && ncls != CLS_NONE;
        if (interior && old_cls != ncls) {
            if (my_slot >= 0) S.list[my_slot] = (tkey << 8) | (uint32_t)ncls;
            if (old_cls != CLS_NONE) atomicSub(&S.cnt[old_cls], 1);
            if (ncls != CLS_NONE) atomicAdd(&S.cnt[ncls], 1);
        }
        if (A && sc) {
            float dn[4] = {0.f, 0.f, 0.f, 0.f}, dold[4] = {0.f, 0.f, 0.f, 0.f};
            if (interior && old_cls != ncls) {
                float Tt = la_temp_at(*A, ta, tb, tz, t_mid);
                la_drate(*A, ncls, Tt, dn, la_vacuum(*A, ncls, tz));
                la_drate(*A, old_cls, Tt, dold, la_vacuum(*A, old_cls, tz));
            }
            for (int j = 0; j < 4; j++) {
                float v = dn[j] - dold[j];
                for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(FULL, v, o);
                G[j] += v;
            }
        }
        unsigned am = __ballot_sync(FULL, append);
        if (append) {
            int ns = nlist + __popc(am & lanemask_lt());
            S.list[ns] = (tkey << 8) | (uint32_t)ncls;
            if (use_pos) S.pos[pos_index(tkey, zw0)] = (uint16_t)ns;
        }
        if (lane == 0) S.nlist = nlist + __popc(am);
        __syncwarp();
        nev++;
        fresh = false;
        // a site that joined the list beyond the staged layers' safe range:
        // re-stage now, before any draw can pick it
        if (__ballot_sync(FULL, append && ((tz - 2 < zw0 && zw0 > 0) || (tz + 3 > zw1 && zw1 < NZ)))) return 1;
    }
}

// One tile for one colour phase of one window: stage, run events from
// t_start to t_start + tau, write back.  Called by the per-colour kernel and
// by the persistent kernel.  COV: the coverage-species rules are compiled in
// (without it every coverage branch folds away).
template <bool LAM, bool COV = false>
__device__ __forceinline__ void process_tile(RepDev *reps, QuadDev *quads, int qid, uint8_t *st_all,
                                             DevStatus *status, uint32_t phase_tag, unsigned int window,
                                             double t_start, LADev *la_all, double *score_all,
                                             const CUtensorMap *tmaps)
{
    TileShared &S = g_tile;
    int lane = threadIdx.x & 31;
    QuadDev Q;
    Q.rep = quads[qid].rep;
    Q.a0 = quads[qid].a0;
    Q.a1 = quads[qid].a1;
    Q.b0 = quads[qid].b0;
    Q.b1 = quads[qid].b1;
    Q.zlo = __ldcg(&quads[qid].zlo);     // widened by neighbouring tiles' atomics
    Q.zhi = __ldcg(&quads[qid].zhi);
    RepDev &Rg = reps[Q.rep];
    RepLocal R = rep_local(Rg);
    if (!COV) R.cov = 0;
    if (!R.active) return;
    if (Q.zhi < Q.zlo) return;   // no event sites in this tile
    // the rate table stays in shared memory while the warp works on tiles of
    // one replica (tables change only between launches); LA staging rewrites
    // the class rates as bounds, so LA tiles reload it
    if (LAM || S.rate_rep != Q.rep) {
        for (int c = lane; c < 64; c += 32) S.rate[c] = Rg.rate[c];
        if (lane < 12) S.spcum[lane / 4][lane % 4] = Rg.spcum[lane / 4][lane % 4];
        __syncwarp();
        if (lane == 0) S.rate_rep = LAM ? -1 : Q.rep;
    }
    __syncwarp();
    uint8_t *st = st_all + R.st_off;
    GLat G{st, R.NA, R.NB, R.NZ, R.pitch};
    const double t_end = t_start + R.tau;
    double t = t_start;
    unsigned int evc = 0;
    unsigned long long nev = 0;
    int hz_lo = 1 << 30, hz_hi = -1;
    int wa = Q.a1 - Q.a0, wb = Q.b1 - Q.b0;
    uint32_t k0 = (uint32_t)R.seed, k1 = (uint32_t)(R.seed >> 32) ^ (0x9E3779B9u * (uint32_t)(Q.rep + 1));
    int zlo = Q.zlo, zhi = Q.zhi;
    int rc = 0;
    const LADev *A = (LAM && la_all[Q.rep].on) ? &la_all[Q.rep] : nullptr;
    const double t_mid = t_start + 0.5 * R.tau;
    double sc[4] = {0.0, 0.0, 0.0, 0.0};
    double *scp = (A && A->score_on) ? sc : nullptr;
    if (lane < 3) S.dcnt[lane] = 0;
    __syncwarp();
    // LA: class rates are bounds at the hottest of the layers [l0, l1]
    auto la_bounds = [&](int l0, int l1) {
        float th = 0.f;
        for (int z = l0 + lane; z <= l1; z += 32)
            th = fmaxf(th, A->tfield ? A->tlayer[z] : la_temp(*A, z, t_mid));
        for (int o = 16; o > 0; o >>= 1) th = fmaxf(th, __shfl_xor_sync(0xffffffffu, th, o));
        for (int c = lane; c < 64; c += 32) S.rate[c] = (c == CLS_ISO) ? 0.f : la_rate(*A, c, th);
        __syncwarp();
    };
    for (int reload = 0;; reload++) {
        if (reload >= NRELOAD) {
            if (lane == 0) set_error(status, DERR_TIMEOUT, qid);
            break;
        }
        int need = zhi - zlo + 5;
        if (need <= WMAX) {
            // stage tile + halo and the layer band in shared memory
            int WZ = min(WMAX, need + 2 * ZMARGIN);
            int zw0 = max(0, zlo - 2 - (WZ - need) / 2);
            int zw1 = min(R.NZ, zw0 + WZ);
            if (zw1 - zw0 < WZ) zw0 = max(0, zw1 - WZ);
            WZ = zw1 - zw0;
            int WA = wa + 2 * HALO, WB = wb + 2 * HALO;
            int lo_a = Q.a0 - HALO;                        // first staged column
            bool inner = lo_a >= 0 && lo_a + WA <= R.NA;
            int ax0 = inner ? (lo_a & ~15) : lo_a;         // column of staged byte 0
            int bx0 = Q.b0 - HALO;
            int nrows = WB * WZ;
            if (tmaps && inner && bx0 >= 0 && bx0 + WB <= R.NB) {
                // no periodic wrap inside the box: one tensor copy per 4 layers
                if (!tma_stage(&tmaps[Q.rep], ax0, bx0, zw0, WZ)) {
                    if (lane == 0) set_error(status, DERR_TIMEOUT, qid);
                    return;
                }
            } else if (inner) {
                // aligned 16-byte chunks, one or two per row: lane -> (row ib,
                // chunk c), eight layers in flight per lane
                int nchunk = ((lo_a - ax0) + WA > 16) ? 2 : 1;
                int c = lane & (nchunk - 1), ib = lane >> (nchunk - 1);
                bool lv = ib < WB;
                const uint8_t *col = st + (int64_t)wrapi(bx0 + ib, R.NB) * R.pitch + ax0 + 16 * c;
                const int64_t zstride = (int64_t)R.NB * R.pitch;
                uint8_t *dst = &S.win[ib * RS + 16 * c];
                for (int iz0 = 0; iz0 < WZ; iz0 += 8) {
                    uint4 v[8];
#pragma unroll
                    for (int u = 0; u < 8; u++)
                        if (lv && iz0 + u < WZ)
                            v[u] = __ldcg(reinterpret_cast<const uint4 *>(col + (int64_t)(zw0 + iz0 + u) * zstride));
#pragma unroll
                    for (int u = 0; u < 8; u++)
                        if (lv && iz0 + u < WZ)
                            *reinterpret_cast<uint4 *>(dst + (iz0 + u) * (WB_MAX * RS)) = v[u];
                }
            } else {
                for (int r = lane; r < nrows; r += 32) {
                    int ib = r % WB, iz = r / WB;
                    const uint8_t *row = st + ((int64_t)(zw0 + iz) * R.NB + wrapi(bx0 + ib, R.NB)) * R.pitch;
                    uint8_t *dst = &S.win[(iz * WB_MAX + ib) * RS];
                    for (int ia = 0; ia < WA; ia++) dst[ia] = __ldcg(&row[wrapi(ax0 + ia, R.NA)]);
                }
            }
            __syncwarp();
            SLat L{ax0, bx0, zw0, R.NZ, st, R.NA, R.NB, R.pitch};
            if (A) la_bounds(zw0, zw1 - 1);
            if (!build_list(L, Q.a0, Q.b0, wa, wb, max(zlo, zw0), min(zhi, zw1 - 1), true, zw0, WZ, R.single != 0, R.cov != 0,
                            R.cov == 2, scp ? A : nullptr, t_mid)) {
                if (lane == 0) set_error(status, DERR_CAPACITY, qid);
                return;
            }
            rc = run_events(L, R, Q, qid, t, t_end, evc, zw0, zw1, true, hz_lo, hz_hi, nev, k0, k1, phase_tag,
                            window, A, t_mid, scp);
            __syncwarp();
            if (rc > 0 && lane == 0) atomicAdd(&status->reloads, 1ull);
        } else {
            // band taller than the staging buffer: run from global memory
            if (lane == 0) atomicAdd(&status->fallback, 1ull);
            // events here may walk the band upwards without re-staging: bound
            // the rates by the top layer (T rises with z)
            if (A) la_bounds(max(0, zlo - 2), R.NZ - 1);
            if (!build_list(G, Q.a0, Q.b0, wa, wb, zlo, zhi, false, 0, 0, R.single != 0, R.cov != 0, R.cov == 2,
                            scp ? A : nullptr, t_mid)) {
                if (lane == 0) set_error(status, DERR_CAPACITY, qid);
                return;
            }
            GLat G2 = G;
            rc = run_events(G2, R, Q, qid, t, t_end, evc, 0, R.NZ, false, hz_lo, hz_hi, nev, k0, k1, phase_tag,
                            window, A, t_mid, scp);
        }
        __syncwarp();
        // z band of the remaining (live) event sites
        int lo = 1 << 30, hi = -1;
        int nl = S.nlist;
        for (int i = lane; i < nl; i += 32) {
            uint32_t en = S.list[i];
            if ((en & 0xFF) == 0) continue;
            int z = (int)(en >> 18);
            lo = min(lo, z);
            hi = max(hi, z);
        }
        for (int o = 16; o > 0; o >>= 1) {
            lo = min(lo, __shfl_xor_sync(0xffffffffu, lo, o));
            hi = max(hi, __shfl_xor_sync(0xffffffffu, hi, o));
        }
        zlo = lo;
        zhi = hi;
        if (rc < 0) {
            if (lane == 0) set_error(status, -rc, qid);
            break;
        }
        if (rc == 0 || zhi < zlo) break;
        __syncwarp();
    }
    __syncwarp();
    for (int o = 16; o > 0; o >>= 1) {
        hz_lo = min(hz_lo, __shfl_xor_sync(0xffffffffu, hz_lo, o));
        hz_hi = max(hz_hi, __shfl_xor_sync(0xffffffffu, hz_hi, o));
    }
    int live = 0;
    for (int c = lane; c < NCLASS; c += 32) live += (c == CLS_NONE) ? 0 : S.cnt[c];
    for (int o = 16; o > 0; o >>= 1) live += __shfl_xor_sync(0xffffffffu, live, o);
    if (lane == 0) {
        quads[qid].zlo = zlo;
        quads[qid].zhi = zhi;
        quads[qid].mc = live;
        // only this tile adds to its count during a launch: a reduction, so
        // the lane does not wait for a read of the old value
        if (nev) atomicAdd(&quads[qid].ev, (int)nev);
        if (scp)
            for (int j = 0; j < 4; j++) atomicAdd(&score_all[4 * Q.rep + j], sc[j]);
        if (A)
            for (int s2 = 0; s2 < 3; s2++)
                if (S.dcnt[s2]) atomicAdd((unsigned long long *)&la_all[Q.rep].cnt[s2], (unsigned long long)(long long)S.dcnt[s2]);
    }
    if (hz_hi >= 0 && lane < 8) {
        // widen the z bands of the neighbouring tiles whose sites changed:
        // lane k takes neighbour k (hz_lo, hz_hi are uniform over the warp),
        // so the eight lookups and reductions are in flight together before
        // the tile publishes its progress
        QuadDev *N = &quads[quads[qid].nbr[lane]];
        atomicMin(&N->zlo, hz_lo);
        atomicMax(&N->zhi, hz_hi);
    }
}

template <bool LAM, bool COV = false>
__global__ void __launch_bounds__(32, 16) k_sl_phase(RepDev *reps, QuadDev *quads, const int *qlist, int nq,
                                                 uint8_t *st_all, DevStatus *status, uint32_t phase_tag,
                                                 LADev *la, double *score, const CUtensorMap *tmaps)
{
    int qi = blockIdx.x;
    if (qi >= nq) return;
    if (threadIdx.x == 0) g_tile.rate_rep = -1;
    tma_barrier_init();
    int qid = qlist[qi];
    const RepDev &R = reps[quads[qid].rep];
    process_tile<LAM, COV>(reps, quads, qid, st_all, status, phase_tag, R.window, R.T0, la, score, tmaps);
}

// Persistent schedule: phases P = ncol*w + colour for windows w = 0..nwin-1 (ncol
// = 4 colours on the square grid of tiles, 3 on the brick tiling).  Warp
// g owns tile i of each colour list for i = g mod G (so at most one tile per
// phase when a colour has <= G tiles) and runs them in increasing P.  A tile of colour c
// may run phase P once each neighbour (all of another colour) has finished
// its last phase before P, i.e. progress[n] >= P - ((c - colour(n)) mod ncol); a
// neighbour cannot start a later phase before this tile publishes P.  All
// waits point to strictly earlier phases and all blocks are co-resident
// (cooperative launch), so the schedule cannot deadlock; every wait is still
// bounded and gives up with DERR_TIMEOUT.  The result equals running the four
// colour launches per window in order.
constexpr long long SPIN_LIMIT_CYCLES = 4000000000LL;   // ~2 s at 2 GHz

template <bool LAM, bool COV = false>
__global__ void __launch_bounds__(32, 16) k_sl_persistent(RepDev *reps, QuadDev *quads, const int *woff,
                                                          const int *wtiles, uint8_t *st_all, DevStatus *status,
                                                          int *progress, int nwin, LADev *la, double *score,
                                                          const CUtensorMap *tmaps, long long spin_limit,
                                                          int hold_tile)
{
    int lane = threadIdx.x & 31;
    if (lane == 0) g_tile.rate_rep = -1;
    tma_barrier_init();
    // this warp's tiles of colour c: wtiles[woff[4 g + c] .. woff[4 g + c + 1])
    const int o0 = woff[4 * blockIdx.x], o1 = woff[4 * blockIdx.x + 1], o2 = woff[4 * blockIdx.x + 2],
              o3 = woff[4 * blockIdx.x + 3], o4 = woff[4 * blockIdx.x + 4];
    for (int c = 0; c < 4; c++) {
        const int kb = c == 0 ? o0 : (c == 1 ? o1 : (c == 2 ? o2 : o3));
        const int ke = c == 0 ? o1 : (c == 1 ? o2 : (c == 2 ? o3 : o4));
        if (ke - kb == 1) {
            const int t = wtiles[kb];
            const int nc = quads[t].ncol;
            if (lane == 0) g_tile.one_ncol[c] = nc;
            if (lane < 8) {
                const int n = quads[t].nbr[lane];
                g_tile.one_nb[c][lane] = (n << 2) | ((c - quads[n].colour + nc) % nc);
            }
        } else if (lane == 0) {
            g_tile.one_ncol[c] = 0;
        }
    }
    __syncwarp();
    // windows in order, colours in order within a window: every wait points
    // to a phase that comes earlier in this order
    for (int w = 0; w < nwin; w++)
        for (int c = 0; c < 4; c++) {
            int kb = c == 0 ? o0 : (c == 1 ? o1 : (c == 2 ? o2 : o3));
            int ke = c == 0 ? o1 : (c == 1 ? o2 : (c == 2 ? o3 : o4));
            const int one_nc = g_tile.one_ncol[c];
            for (int k = kb; k < ke; k++) {
                int t = wtiles[k];
                const int ncol = one_nc ? one_nc : quads[t].ncol;
                const int P = ncol * w + c;
                // lane 8 reads the error word while lanes 0..7 poll, so a
                // phase whose flags are already set costs one round trip
                int bad = lane == 8 ? *(volatile int *)&status->error : 0;
                if (lane < 8) {
                    int n, need;
                    if (one_nc) {
                        const int v = g_tile.one_nb[c][lane];
                        n = v >> 2;
                        need = P - (v & 3);
                    } else {
                        n = quads[t].nbr[lane];
                        need = P - (c - quads[n].colour + ncol) % ncol;
                    }
                    long long t0 = clock64();
                    volatile int *pr = progress + n;
                    volatile int *err = &status->error;
                    // tight poll (one L2 round trip per check; a sleep between
                    // checks oversleeps the flag and lengthens every phase)
                    while (*pr < need) {
                        if (*err) {
                            bad = 1;
                            break;
                        }
                        if (clock64() - t0 > spin_limit) {
                            set_error(status, DERR_TIMEOUT, t);
                            bad = 1;
                            break;
                        }
                    }
                }
                __syncwarp();
                __threadfence();                                // acquire: neighbours' writes before their flag
                if (__any_sync(0xffffffffu, bad != 0)) return;
                const RepDev &R = reps[quads[t].rep];
                process_tile<LAM, COV>(reps, quads, t, st_all, status, (uint32_t)c, R.window + (unsigned)w,
                                       R.T0 + (double)w * R.tau, la, score, tmaps);
                __threadfence();                                // release: each lane's writes reach L2 ...
                __syncwarp();                                   // ... before lane 0 publishes the flag
                if (lane == 0 && t != hold_tile) atomicExch(progress + t, P);
            }
        }
}

// End of a window: advance the replica clock, apply the exit conditions.
__global__ void k_window_end(RepDev *reps, QuadDev *quads, int nwin, LADev *la)
{
    RepDev &R = reps[blockIdx.x];
    long long s = 0, e = 0;
    int nqt = R.nqa * R.nqb;
    for (int i = threadIdx.x; i < nqt; i += blockDim.x) {
        QuadDev &q = quads[R.quad_base + i];
        s += q.mc;
        e += q.ev;
        q.ev = 0;
    }
    __shared__ long long sh[256], she[256];
    sh[threadIdx.x] = s;
    she[threadIdx.x] = e;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if ((int)threadIdx.x < o) {
            sh[threadIdx.x] += sh[threadIdx.x + o];
            she[threadIdx.x] += she[threadIdx.x + o];
        }
        __syncthreads();
    }
    if (threadIdx.x == 0) R.events += (unsigned long long)she[0];
    if (threadIdx.x == 0) {
        R.mc_count = sh[0];
        if (!R.active) return;
        R.T0 += (double)nwin * R.tau;
        unsigned wold = R.window;
        R.window += (unsigned)nwin;
        if (la && la[blockIdx.x].on && la[blockIdx.x].liquid_weighting) {
            LADev &A = la[blockIdx.x];
            long long liq[3], sum = 0, crys = 0, init = 0;
            for (int s = 0; s < 3; s++) {
                liq[s] = A.init_cnt[s] - A.cnt[s];
                if (liq[s] < 0) liq[s] = 0;
                sum += liq[s];
                crys += A.cnt[s];
                init += A.init_cnt[s];
            }
            if (R.window / LA_PHASE != wold / LA_PHASE)
                for (int s = 0; s < 3; s++) A.xliq[s] = sum > 0 ? (float)((double)liq[s] / (double)sum) : 0.f;
            // LaserAnnealing main.f:714-723: stop once more sites are occupied
            // than before the melt
            if (crys > init) {
                R.active = 0;
                R.stop_reason = 4;
                return;
            }
        }
        if (R.mc_count <= 20) {
            R.active = 0;
            R.stop_reason = 1;
        } else if ((long long)R.events >= R.ev_max) {
            R.active = 0;
            R.stop_reason = 2;
        } else if (R.T0 >= R.t_max) {
            R.active = 0;
            R.stop_reason = 3;
        }
    }
}

// LR gradient of E[f] from the FP64 scores (the backward step of the LA
// score): grad_j = 1/(n-1) sum_i (f_i - mean f) S_ij, which equals the mean of
// (f_i - b_i) S_ij with the leave-one-out baseline b_i and is unbiased; se_j
// is its standard error.  One block, FP64.
__global__ void k_lr_grad(const double *score, const double *f, int n, int use_b, double *out)
{
    __shared__ double sh[256];
    int tid = threadIdx.x;
    auto block_sum = [&](double v) {
        sh[tid] = v;
        __syncthreads();
        for (int o = blockDim.x / 2; o > 0; o >>= 1) {
            if (tid < o) sh[tid] += sh[tid + o];
            __syncthreads();
        }
        double r = sh[0];
        __syncthreads();
        return r;
    };
    double fs = 0.0;
    for (int i = tid; i < n; i += blockDim.x) fs += f[i];
    double fbar = use_b ? block_sum(fs) / n : 0.0;
    double scale = (use_b && n > 1) ? (double)n / (double)(n - 1) : 1.0;
    for (int j = 0; j < 4; j++) {
        double s1 = 0.0, s2 = 0.0;
        for (int i = tid; i < n; i += blockDim.x) {
            double x = scale * (f[i] - fbar) * score[4 * i + j];
            s1 += x;
            s2 += x * x;
        }
        s1 = block_sum(s1);
        s2 = block_sum(s2);
        if (tid == 0) {
            double m = s1 / n;
            double var = n > 1 ? fmax(0.0, (s2 - n * m * m) / (n - 1)) : 0.0;
            out[j] = m;
            out[4 + j] = sqrt(var / n);
        }
    }
}

// Causal step of the LR gradient: for increments df of the observable over
// the last segment, acc_i += (df_i - b_i) S_i with S_i the replica's score
// so far and b_i the leave-one-out mean of df (unbiased: b_i is independent
// of replica i, and E[S_i] = 0).  One block, FP64.
__global__ void k_lr_step(const double *score, const double *df, int n, double *acc)
{
    __shared__ double sh[256];
    int tid = threadIdx.x;
    double fs = 0.0;
    for (int i = tid; i < n; i += blockDim.x) fs += df[i];
    sh[tid] = fs;
    __syncthreads();
    for (int o = blockDim.x / 2; o > 0; o >>= 1) {
        if (tid < o) sh[tid] += sh[tid + o];
        __syncthreads();
    }
    const double tot = sh[0];
    for (int i = tid; i < n; i += blockDim.x) {
        double b = n > 1 ? (tot - df[i]) / (double)(n - 1) : 0.0;
        double w = df[i] - b;
        for (int j = 0; j < 4; j++) acc[4 * i + j] += w * score[4 * i + j];
    }
}

// ---- frame writer support: order-preserving selection of listed sites ----
// kind 0: atoms with coordination <= 3 (the main I*.xyz list,
// WriteMolMolXYZFile.f:171-215); kind 1: voids (empty, coordination 4, the
// O lines and _v.xyz, :216-260).  Kinds 2 and 3 are the same lists in
// coverage mode: covered sites join the main list (the H / Cl lines of
// :176-178) and covered voids the voids.  Sites are visited in layer, row,
// column order, which is the reference's z, y, x scan order.
__device__ __forceinline__ bool frame_pick(uint8_t s, int kind)
{
    if (s == 0 || s == WALL) return false;
    int sp = sp_of(s), co = co_of(s);
    if (kind == 0) return sp != 0 && co <= 3;
    if (kind == 1) return sp == 0 && co == 4;
    if (kind == 2) return sp == COVSP || (sp != 0 && co <= 3);
    return (sp == 0 || sp == COVSP) && co == 4;
}

// The padded lattice is read as 16-byte units (row-major, so unit order is
// the reference's z, y, x order); a block takes FRAME_UNITS consecutive
// units, four per thread.  Padding bytes and non-site bytes are 0.
constexpr int FRAME_UNITS = 1024;

__device__ __forceinline__ unsigned frame_mask(uint4 v, int kind)
{
    const uint8_t *by = reinterpret_cast<const uint8_t *>(&v);
    unsigned m = 0;
#pragma unroll
    for (int k = 0; k < 16; k++) m |= frame_pick(by[k], kind) ? (1u << k) : 0u;
    return m;
}

__global__ void k_frame_count(const RepDev *reps, int rep, const uint8_t *st_all, int kind, unsigned int *counts)
{
    const RepDev &R = reps[rep];
    const uint4 *st = reinterpret_cast<const uint4 *>(st_all + R.st_off);
    int64_t nu = (int64_t)R.NZ * R.NB * (R.pitch / 16);
    int64_t u0 = (int64_t)blockIdx.x * FRAME_UNITS + 4 * threadIdx.x;
    unsigned int cnt = 0;
#pragma unroll
    for (int j = 0; j < 4; j++)
        if (u0 + j < nu) cnt += __popc(frame_mask(__ldcs(st + u0 + j), kind));
    for (int o = 16; o > 0; o >>= 1) cnt += __shfl_xor_sync(0xffffffffu, cnt, o);
    __shared__ unsigned int sh;
    if (threadIdx.x == 0) sh = 0;
    __syncthreads();
    if ((threadIdx.x & 31) == 0) atomicAdd(&sh, cnt);
    __syncthreads();
    if (threadIdx.x == 0) counts[blockIdx.x] = sh;
}

// ordered compaction: block-wide exclusive scan of the per-thread counts
__global__ void k_frame_write(const RepDev *reps, int rep, const uint8_t *st_all, int kind,
                              const unsigned long long *offsets, uint32_t *out)
{
    const RepDev &R = reps[rep];
    const uint4 *st = reinterpret_cast<const uint4 *>(st_all + R.st_off);
    const int upr = R.pitch / 16;                               // units per row
    int64_t nu = (int64_t)R.NZ * R.NB * upr;
    int64_t u0 = (int64_t)blockIdx.x * FRAME_UNITS + 4 * threadIdx.x;
    unsigned m[4];
    unsigned int cnt = 0;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        m[j] = u0 + j < nu ? frame_mask(__ldcs(st + u0 + j), kind) : 0u;
        cnt += __popc(m[j]);
    }
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    unsigned int x = cnt;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
        unsigned int y = __shfl_up_sync(0xffffffffu, x, o);
        if (lane >= o) x += y;
    }
    __shared__ unsigned int wsum[32];
    if (lane == 31) wsum[wid] = x;
    __syncthreads();
    unsigned int before = x - cnt;
    for (int w = 0; w < wid; w++) before += wsum[w];
    unsigned long long pos = offsets[blockIdx.x] + before;
#pragma unroll
    for (int j = 0; j < 4; j++) {
        unsigned mm = m[j];
        int64_t row = (u0 + j) / upr;
        int abase = 16 * (int)((u0 + j) - row * upr);
        while (mm) {
            int k = __ffs(mm) - 1;
            mm &= mm - 1;
            out[pos++] = (uint32_t)(row * R.NA + abase + k);
        }
    }
}

// ------------------------------------------------------------ host side
// named profiler range for the duration of a scope
struct NvtxRange {
    explicit NvtxRange(const char *name) { nvtxRangePushA(name); }
    ~NvtxRange() { nvtxRangePop(); }
};

thread_local std::string g_err;

int fail(int code, const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof buf, fmt, ap);
    va_end(ap);
    g_err = buf;
    return code;
}

#define CK(call)                                                                            \
    do {                                                                                    \
        cudaError_t e_ = (call);                                                            \
        if (e_ != cudaSuccess) return fail(MKS_ERR_CUDA, "%s: %s", #call, cudaGetErrorString(e_)); \
    } while (0)

struct RepHost {
    mks_config cfg;
    int NA, NB, NZ, pitch;
    int nqa, nqb, quad_base;
    int qshift = 0;             // brick tiling: shift of the odd tile rows (columns)
    int width = 8;              // tile width (sites) of this replica's tiling
    int64_t st_off;
    double ptransE[3 * 4096];
    double ptransD[9];
    double ptransAbs[9] = {0};  // [coverage species][coor-1] (SetProbability.f:121-131)
    double ptransDes[9] = {0};  // [coverage species][coor-1] (:132-140)
    bool rates_set = false;
    int64_t t_layer_off = -1;   // offset in d_tlayer once a temperature field is loaded
};

}  // namespace

struct mks_handle {
    std::vector<RepHost> reps;
    std::vector<QuadDev> quads_h;
    std::vector<int> color_list_h[4];
    int64_t st_bytes = 0;
    uint8_t *d_st = nullptr;
    RepDev *d_reps = nullptr;
    QuadDev *d_quads = nullptr;
    int *d_clist[4] = {nullptr, nullptr, nullptr, nullptr};
    DevStatus *d_status = nullptr;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    cudaGraphExec_t graph_exec = nullptr;
    int graph_windows = 0;
    int tile_width = 8;
    int *d_progress = nullptr;
    int *d_woff = nullptr, *d_wtiles = nullptr;   // persistent schedule (upload_tiles)
    long long spin_limit = SPIN_LIMIT_CYCLES;     // bounded neighbour waits (cycles)
    int hold_tile = -1;                           // failure injection: a tile that never publishes
    CUtensorMap *d_tmaps = nullptr;               // one per replica for TMA staging; null: plain loads
    uint8_t *d_st2 = nullptr;                     // second lattice buffer (mks_prefetch_state)
    CUtensorMap *d_tmaps2 = nullptr;
    cudaStream_t copy_stream = nullptr;
    cudaEvent_t ev_copy = nullptr, ev_swap = nullptr;
    bool prefetched = false;
    uint16_t *d_tfield = nullptr;                 // LA static temperatures, lattice layout
    float *d_tlayer = nullptr;                    // their maximum per layer (all replicas)
    LADev *d_la = nullptr;
    double *d_score = nullptr;
    int la_on = 0;
    int64_t la_window = 0;
    double *d_lr = nullptr;      // f values and result of mks_batch_lr_grad
    double *d_lr_acc = nullptr;  // causal LR sums per replica (4 each), then ones and the result
    int coop_grid = 0;
    bool any_cov = false;        // a replica has a coverage species: the COV kernels run
    int schedule = 1;            // 1 persistent dataflow kernel, 0 one launch per colour phase
    uint32_t phase_counter = 0;
    int ncolour = 4;             // most colours of a replica's tiling: 4 square grid, 3 brick
    int colours_req = 0;         // 0: brick for every replica that admits it; 4: square grid for all
    int64_t last_kernels = 0, last_graphs = 0, last_phase_launches = 0;
    double last_ms = 0.0;
    double time_acc = 0.0;
    unsigned char *noalloc_scratch = nullptr;  // device address of the mks_replay_noalloc array (set at creation)
    // PtransZig < 1: the explicit-neighbour engine (stacking.cu) runs the
    // lattice; the initializers still build it in compact form, expanded at
    // the first call that needs the explicit form (stk_dirty)
    mks_stk::State *stk = nullptr;
    bool stk_dirty = false;
};

namespace {

void rate_tables(const RepHost &r, RepDev &d)
{
    for (int c = 0; c < 64; c++) d.rate[c] = 0.f;
    const bool cov = r.cfg.ncov > 0;
    const double *pD = r.ptransD;
    for (int co = 1; co <= 3; co++) {
        double p1 = pD[co - 1], p2 = pD[3 + co - 1], p3 = pD[6 + co - 1];
        double dep = p1 + p2 + p3;
        // empty site: deposition of any species or absorption of a coverage
        // species, one rate (Get_Prob.f:155-204; the absorption sum runs over
        // the species in order, as SUM(PtransAbs(:,Coor)) does)
        const double a1 = r.ptransAbs[co - 1], a2 = r.ptransAbs[3 + co - 1];
        double tot = dep + (cov ? (a1 + a2) + r.ptransAbs[6 + co - 1] : 0.0);
        int cls = co == 1 ? CLS_C1 : (co == 2 ? CLS_C2 : CLS_C3);
        d.rate[cls] = (float)tot;
        d.spcum[co - 1][0] = tot > 0 ? (float)(p1 / tot) : 1.f;
        d.spcum[co - 1][1] = tot > 0 ? (float)((p1 + p2) / tot) : 1.f;
        d.spcum[co - 1][2] = (tot > 0 && cov) ? (float)(dep / tot) : 1.f;
        d.spcum[co - 1][3] = (tot > 0 && cov) ? (float)((dep + a1) / tot) : 1.f;
        if (cov) d.rate[CLS_D1 + co - 1] = (float)r.ptransDes[co - 1];   // Get_Prob.f:114
        if (r.cfg.ncov == 2) d.rate[CLS_D2 + co - 1] = (float)r.ptransDes[3 + co - 1];
    }
    d.rate[CLS_C1D] = 1.e-8f;   // Get_Prob.f:183
    d.rate[CLS_C1I] = 1.e-6f;   // Get_Prob_Ini.f:104
    d.rate[CLS_ISO] = 0.f;      // dynamic: 1e5 x tile rate (Get_Prob.f:305)
    if (r.cfg.ncov == 2) {
        // PE(1, n1, 0, 0, c1, c2, 0), Get_Prob.f:309-312
        for (int n1 = 1; n1 <= 3; n1++)
            for (int c1 = 0; c1 <= 4 - n1; c1++)
                for (int c2 = 0; c1 + c2 <= 4 - n1; c2++)
                    d.rate[CLS_COV0 + cov2_census_index(n1, c1, c2)] =
                        (float)r.ptransE[n1 * 1024 + c1 * 16 + c2 * 4];
        return;
    }
    if (cov) {
        // PE(NSiC, n1, n2, 0, c, 0, 0), Get_Prob.f:309-312
        for (int sp = 1; sp <= 2; sp++)
            for (int n1 = 0; n1 <= 3; n1++)
                for (int n2 = 0; n1 + n2 <= 3; n2++) {
                    int t = n1 + n2;
                    if (t < 1) continue;
                    for (int c = 0; c <= 4 - t; c++) {
                        double v = r.ptransE[(sp - 1) * 4096 + n1 * 1024 + n2 * 256 + c * 16];
                        d.rate[CLS_COV0 + (sp - 1) * NCOVCENSUS + cov_census_index(n1, n2, c)] = (float)v;
                    }
                }
        return;
    }
    for (int sp = 1; sp <= 3; sp++)
        for (int n1 = 0; n1 <= 3; n1++)
            for (int n2 = 0; n2 <= 3; n2++)
                for (int n3 = 0; n3 <= 3; n3++) {
                    int t = n1 + n2 + n3;
                    if (t < 1 || t > 3) continue;
                    double v = r.ptransE[(sp - 1) * 4096 + n1 * 1024 + n2 * 256 + n3 * 64];
                    d.rate[CLS_OCC0 + (sp - 1) * NCENSUS + census_index(n1, n2, n3)] = (float)v;
                }
}

int check_config(const mks_config &c)
{
    if (c.lenx <= 0 || c.leny <= 0 || c.lenz <= 0 || c.lenx % 12 || c.leny % 12 || c.lenz % 3)
        return fail(MKS_ERR_ARG, "box %dx%dx%d: LenX, LenY must be multiples of 12 and LenZ of 3", c.lenx, c.leny,
                    c.lenz);
    if (c.lenx / 6 < 16 || c.leny / 6 < 16)
        return fail(MKS_ERR_ARG, "box side %d/%d too small (needs >= 96 grid units)", c.lenx, c.leny);
    if (c.ncrystal < 1 || c.ncrystal > 3) return fail(MKS_ERR_ARG, "NCrystal must be 1..3");
    if (c.ncov < 0 || c.ncov > 2)
        return fail(MKS_ERR_UNSUPPORTED, "NCov=%d: the GPU engine holds two coverage species at most", c.ncov);
    if (c.ncov == 2 && c.ncrystal != 1)
        return fail(MKS_ERR_UNSUPPORTED, "two coverage species need NCrystal = 1 (the rate classes of their census)");
    if (c.ncov == 2 && (c.list_cov[1] <= 0 || c.list_cov[1] >= 113 || c.list_cov[1] == c.list_cov[0]))
        return fail(MKS_ERR_ARG, "second coverage species atomic number %d", c.list_cov[1]);
    if (c.ncov == 1 && c.ncrystal > 2)
        return fail(MKS_ERR_UNSUPPORTED, "a coverage species needs NCrystal <= 2 (species value 3 marks covered sites)");
    if (c.ncov == 1 && (c.list_cov[0] <= 0 || c.list_cov[0] >= 113))
        return fail(MKS_ERR_ARG, "coverage species atomic number %d", c.list_cov[0]);
    if (!(c.ptrans_zig >= 0.0 && c.ptrans_zig <= 1.0)) return fail(MKS_ERR_ARG, "PtransZig=%g outside [0, 1]", c.ptrans_zig);
    if (c.ptrans_zig != 1.0 && c.ncov)
        return fail(MKS_ERR_UNSUPPORTED, "PtransZig=%g with a coverage species: arm-chair stacking runs without coverage",
                    c.ptrans_zig);
    if (c.explicit_nn != 0 && c.explicit_nn != 1) return fail(MKS_ERR_ARG, "explicit_nn=%d is not 0 or 1", c.explicit_nn);
    if (c.explicit_nn && c.ncov)
        return fail(MKS_ERR_UNSUPPORTED, "the explicit-neighbour engine runs without coverage species");
    return 0;
}

// even number of tiles per side
// even number of tiles along a side of n sites, each about `width` wide
// (at least 4: the write ring of one tile and the read halo of the next
// same-colour tile must not meet) and at most QMAX
int upload_reps(mks_handle *h, const std::vector<RepDev> &d)
{
    CK(cudaMemcpyAsync(h->d_reps, d.data(), sizeof(RepDev) * d.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int download_reps(mks_handle *h, std::vector<RepDev> &d)
{
    d.resize(h->reps.size());
    CK(cudaMemcpyAsync(d.data(), h->d_reps, sizeof(RepDev) * d.size(), cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int read_status(mks_handle *h, DevStatus &s)
{
    CK(cudaMemcpyAsync(&s, h->d_status, sizeof s, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int read_status(mks_handle *h, DevStatus &s);

int rescan(mks_handle *h)
{
    NvtxRange nr("mks_rescan");
    if (h->stk) h->stk_dirty = true;      // a new compact lattice: expand it before the next stacking call
    int nq = (int)h->quads_h.size();
    k_band_init<<<std::min(1024, (nq + 255) / 256), 256, 0, h->stream>>>(h->d_quads, 0, nq);
    for (size_t i = 0; i < h->reps.size(); i++) {
        const RepHost &r = h->reps[i];
        int64_t nu = (int64_t)r.NZ * r.NB * (r.pitch / 16);
        int blocks = (int)std::min<int64_t>(152 * 16, (nu + 255) / 256);
        k_band_scan<<<blocks, 256, 0, h->stream>>>(h->d_reps, (int)i, h->d_quads, h->d_st, h->d_status);
    }
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    DevStatus s;
    int rc = read_status(h, s);
    if (rc) return rc;
    if (s.error) return fail(MKS_ERR_INVARIANT, "lattice check failed in tile %d (species above NCrystal?)", s.err_quad);
    return 0;
}

// class histograms of replicas [r0, r1) into hist (zeroed by the caller)
void class_hist(mks_handle *h, int r0, int r1, unsigned long long *hist)
{
    int q0 = h->reps[r0].quad_base;
    int q1 = r1 < (int)h->reps.size() ? h->reps[r1].quad_base : (int)h->quads_h.size();
    int nb = std::min(q1 - q0, 8192);
    if (nb > 0) k_class_hist<<<nb, 128, 0, h->stream>>>(h->d_reps, h->d_quads, q0, q1, r0, h->d_st, hist);
}

// cut every replica's (a,b) plane into tiles of about `width` sites
// The tiles of every replica (mks_tiling::layout): the brick tiling of three
// colours where a replica admits it and colours_req allows, else the square
// grid of four.
void partition(mks_handle *h)
{
    h->quads_h.clear();
    for (int c = 0; c < 4; c++) h->color_list_h[c].clear();
    h->ncolour = 0;
    for (size_t i = 0; i < h->reps.size(); i++) {
        RepHost &r = h->reps[i];
        const mks_tiling::Layout L = mks_tiling::layout(r.NA, r.NB, r.width, h->colours_req != 4);
        h->ncolour = std::max(h->ncolour, L.ncol);
        r.nqa = L.nqa;
        r.nqb = L.nqb;
        r.qshift = L.shift;
        r.quad_base = (int)h->quads_h.size();
        for (const mks_tiling::Tile &t : L.tiles) {
            QuadDev q;
            q.rep = (int)i;
            q.a0 = t.a0;
            q.a1 = t.a1;
            q.b0 = t.b0;
            q.b1 = t.b1;
            q.zlo = 1 << 30;
            q.zhi = -1;
            q.mc = 0;
            q.qa = t.qa;
            q.qb = t.qb;
            q.colour = t.colour;
            q.ncol = L.ncol;
            q.ev = 0;
            for (int k = 0; k < 8; k++) q.nbr[k] = r.quad_base + t.nbr[k];
            h->color_list_h[q.colour].push_back((int)h->quads_h.size());
            h->quads_h.push_back(q);
        }
    }
}

int upload_tiles(mks_handle *h)
{
    cudaFree(h->d_quads);
    h->d_quads = nullptr;
    CK(cudaMalloc(&h->d_quads, sizeof(QuadDev) * h->quads_h.size()));
    CK(cudaMemcpyAsync(h->d_quads, h->quads_h.data(), sizeof(QuadDev) * h->quads_h.size(), cudaMemcpyHostToDevice,
                       h->stream));
    for (int c = 0; c < 4; c++) {
        cudaFree(h->d_clist[c]);
        h->d_clist[c] = nullptr;
        size_t nb = sizeof(int) * std::max<size_t>(1, h->color_list_h[c].size());
        CK(cudaMalloc(&h->d_clist[c], nb));
        if (!h->color_list_h[c].empty())
            CK(cudaMemcpyAsync(h->d_clist[c], h->color_list_h[c].data(), sizeof(int) * h->color_list_h[c].size(),
                               cudaMemcpyHostToDevice, h->stream));
    }
    cudaFree(h->d_progress);
    h->d_progress = nullptr;
    CK(cudaMalloc(&h->d_progress, sizeof(int) * h->quads_h.size()));
    // resident grid of the persistent kernel (cooperative launch)
    int dev = 0, nsm = 0, per_sm = 0;
    CK(cudaGetDevice(&dev));
    CK(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    int per_sm_la = 0, per_sm_cov = 0;
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_sl_persistent<false>, 32, 0));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_la, k_sl_persistent<true>, 32, 0));
    CK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm_cov, k_sl_persistent<false, true>, 32, 0));
    per_sm = std::min(per_sm, std::min(per_sm_la, per_sm_cov));
    size_t maxc = 0;
    for (int c = 0; c < 4; c++) maxc = std::max(maxc, h->color_list_h[c].size());
    h->coop_grid = (int)std::min<int64_t>((int64_t)nsm * std::max(per_sm, 1), (int64_t)std::max<size_t>(1, maxc));
    // persistent schedule: tile i of colour list c goes to warp i mod G, so a
    // warp holds at most ceil(n_c / G) tiles of a colour, and neighbouring
    // warps hold neighbouring tiles
    int G = h->coop_grid;
    std::vector<int> woff(4 * (size_t)G + 1, 0), wtiles;
    wtiles.reserve(h->quads_h.size());
    for (int g = 0; g < G; g++)
        for (int c = 0; c < 4; c++) {
            woff[4 * (size_t)g + c] = (int)wtiles.size();
            const std::vector<int> &L = h->color_list_h[c];
            for (size_t i = (size_t)g; i < L.size(); i += (size_t)G) wtiles.push_back(L[i]);
        }
    woff[4 * (size_t)G] = (int)wtiles.size();
    cudaFree(h->d_woff);
    cudaFree(h->d_wtiles);
    h->d_woff = h->d_wtiles = nullptr;
    CK(cudaMalloc(&h->d_woff, sizeof(int) * woff.size()));
    CK(cudaMalloc(&h->d_wtiles, sizeof(int) * std::max<size_t>(1, wtiles.size())));
    CK(cudaMemcpyAsync(h->d_woff, woff.data(), sizeof(int) * woff.size(), cudaMemcpyHostToDevice, h->stream));
    if (!wtiles.empty())
        CK(cudaMemcpyAsync(h->d_wtiles, wtiles.data(), sizeof(int) * wtiles.size(), cudaMemcpyHostToDevice,
                           h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

// One TMA tensor map per replica over its lattice: dims (pitch, NB, NZ)
// bytes, box (32, WB_MAX, TMA_BZ).  Left unset (the tiles then stage with
// plain loads) if the driver has no encoder or a replica is narrower than a
// box row.
typedef CUresult (*EncodeTiledFn)(CUtensorMap *, CUtensorMapDataType, cuuint32_t, void *, const cuuint64_t *,
                                  const cuuint64_t *, const cuuint32_t *, const cuuint32_t *, CUtensorMapInterleave,
                                  CUtensorMapSwizzle, CUtensorMapL2promotion, CUtensorMapFloatOOBfill);

int make_tensor_maps(mks_handle *h, uint8_t *base, CUtensorMap **out)
{
    cudaFree(*out);
    *out = nullptr;
    for (const RepHost &r : h->reps)
        if (r.pitch < RS || r.NB < WB_MAX || r.NZ < TMA_BZ) return 0;
    void *fn = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &fn, 12000, cudaEnableDefault, &q) != cudaSuccess ||
        q != cudaDriverEntryPointSuccess || !fn) {
        cudaGetLastError();
        return 0;
    }
    EncodeTiledFn enc = (EncodeTiledFn)fn;
    std::vector<CUtensorMap> maps(h->reps.size());
    for (size_t i = 0; i < h->reps.size(); i++) {
        const RepHost &r = h->reps[i];
        cuuint64_t dims[3] = {(cuuint64_t)r.pitch, (cuuint64_t)r.NB, (cuuint64_t)r.NZ};
        cuuint64_t strides[2] = {(cuuint64_t)r.pitch, (cuuint64_t)r.NB * (cuuint64_t)r.pitch};
        cuuint32_t box[3] = {(cuuint32_t)RS, (cuuint32_t)WB_MAX, (cuuint32_t)TMA_BZ};
        cuuint32_t es[3] = {1, 1, 1};
        if (enc(&maps[i], CU_TENSOR_MAP_DATA_TYPE_UINT8, 3, base + r.st_off, dims, strides, box, es,
                CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE, CU_TENSOR_MAP_L2_PROMOTION_L2_128B,
                CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE) != CUDA_SUCCESS)
            return 0;
    }
    CK(cudaMalloc(out, sizeof(CUtensorMap) * maps.size()));
    CK(cudaMemcpy(*out, maps.data(), sizeof(CUtensorMap) * maps.size(), cudaMemcpyHostToDevice));
    return 0;
}

}  // namespace

// ---- mks_replay_noalloc: the replay kernel fed from a library-owned array ----
// Layout of the array: bytes [0, 8) the kernel's progress counter, bytes
// [256, 256 + 16 * MKS_REPLAY_NOALLOC_MAX) the staged events.  Every GPU that
// loads this library holds the array until the process exits.
static __device__ __align__(256) unsigned char g_replay_scratch[256 + sizeof(mks_event) * MKS_REPLAY_NOALLOC_MAX];

namespace {

// Device address of g_replay_scratch on the current device.  In host code the
// symbol itself is only a stand-in for the device array, never a device
// address.  Called by create_impl with the handle's device current, outside
// any stream capture, so each handle carries the address of the array in its
// own context (a context created again after a device reset reloads the
// module, and its handles look the address up afresh).
int noalloc_lookup(unsigned char **out)
{
    void *p = nullptr;
    cudaError_t e = cudaGetSymbolAddress(&p, g_replay_scratch);
    if (e != cudaSuccess) return fail(MKS_ERR_CUDA, "cudaGetSymbolAddress: %s", cudaGetErrorString(e));
    *out = static_cast<unsigned char *>(p);
    return 0;
}

int create_impl(const mks_config *cfgs, int n, mks_handle **out)
{
    if (!cfgs || n <= 0 || !out) return fail(MKS_ERR_ARG, "bad arguments");
    int ndev = 0;
    if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0)
        return fail(MKS_ERR_CUDA, "no CUDA device: the GB300 engine has no CPU path");
    mks_handle *h = new mks_handle();
    int64_t off = 0;
    for (int i = 0; i < n; i++) {
        int rc = check_config(cfgs[i]);
        if (rc) {
            delete h;
            return rc;
        }
        RepHost r;
        r.cfg = cfgs[i];
        r.NA = cfgs[i].lenx / 6;
        r.NB = cfgs[i].leny / 6;
        r.NZ = cfgs[i].lenz / 3 + 1;
        r.pitch = (r.NA + 15) & ~15;
        r.st_off = off;
        off += (int64_t)r.NZ * r.NB * r.pitch;
        off = (off + 255) & ~(int64_t)255;
        memset(r.ptransE, 0, sizeof r.ptransE);
        memset(r.ptransD, 0, sizeof r.ptransD);
        h->reps.push_back(r);
    }
    h->st_bytes = off;
    for (int i = 0; i < n; i++)
        if ((cfgs[i].ptrans_zig != 1.0 || cfgs[i].explicit_nn) && n != 1) {
            delete h;
            return fail(MKS_ERR_UNSUPPORTED,
                        "the explicit-neighbour engine (PtransZig < 1, explicit_nn) runs in single-replica handles");
        }
    partition(h);
    auto cleanup_fail = [&](const char *what, cudaError_t e) {
        fail(MKS_ERR_CUDA, "%s: %s", what, cudaGetErrorString(e));
        mks_destroy(h);
        return MKS_ERR_CUDA;
    };
    cudaError_t e;
    if ((e = cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking)) != cudaSuccess) return cleanup_fail("stream", e);
    if (noalloc_lookup(&h->noalloc_scratch)) {
        mks_destroy(h);
        return MKS_ERR_CUDA;
    }
    if ((e = cudaEventCreate(&h->ev0)) != cudaSuccess) return cleanup_fail("event", e);
    if ((e = cudaEventCreate(&h->ev1)) != cudaSuccess) return cleanup_fail("event", e);
    if ((e = cudaMalloc(&h->d_st, (size_t)h->st_bytes)) != cudaSuccess) return cleanup_fail("lattice allocation", e);
    if ((e = cudaMemsetAsync(h->d_st, 0, (size_t)h->st_bytes, h->stream)) != cudaSuccess) return cleanup_fail("memset", e);
    if ((e = cudaMalloc(&h->d_reps, sizeof(RepDev) * n)) != cudaSuccess) return cleanup_fail("alloc", e);
    if ((e = cudaMalloc(&h->d_status, sizeof(DevStatus))) != cudaSuccess) return cleanup_fail("alloc", e);
    if ((e = cudaMalloc(&h->d_la, sizeof(LADev) * n)) != cudaSuccess) return cleanup_fail("alloc", e);
    if ((e = cudaMemsetAsync(h->d_la, 0, sizeof(LADev) * n, h->stream)) != cudaSuccess) return cleanup_fail("memset", e);
    if ((e = cudaMalloc(&h->d_score, sizeof(double) * 4 * n)) != cudaSuccess) return cleanup_fail("alloc", e);
    if ((e = cudaMemsetAsync(h->d_score, 0, sizeof(double) * 4 * n, h->stream)) != cudaSuccess)
        return cleanup_fail("memset", e);
    if ((e = cudaMemsetAsync(h->d_status, 0, sizeof(DevStatus), h->stream)) != cudaSuccess) return cleanup_fail("memset", e);
    {
        int rc_t = upload_tiles(h);
        if (!rc_t) rc_t = make_tensor_maps(h, h->d_st, &h->d_tmaps);
        if (rc_t) {
            mks_destroy(h);
            return rc_t;
        }
    }
    std::vector<RepDev> d(n);
    for (int i = 0; i < n; i++) {
        memset(&d[i], 0, sizeof(RepDev));
        const RepHost &r = h->reps[i];
        d[i].st_off = r.st_off;
        d[i].NA = r.NA;
        d[i].NB = r.NB;
        d[i].NZ = r.NZ;
        d[i].pitch = r.pitch;
        d[i].nqa = r.nqa;
        d[i].nqb = r.nqb;
        d[i].qshift = r.qshift;
        d[i].quad_base = r.quad_base;
        d[i].tau = 1e-6;
        d[i].T0 = 0.0;
        d[i].t_max = 1e300;
        d[i].ev_max = (long long)9e18;
        d[i].seed = r.cfg.seed;
        d[i].active = 1;
        d[i].single = r.cfg.ncrystal == 1 && r.cfg.ncov == 0;
        d[i].cov = r.cfg.ncov;
        if (d[i].cov) h->any_cov = true;
        rate_tables(r, d[i]);
    }
    int rc = upload_reps(h, d);
    if (rc) {
        mks_destroy(h);
        return rc;
    }
    if (n == 1 && (cfgs[0].ptrans_zig != 1.0 || cfgs[0].explicit_nn)) {
        std::string err;
        rc = mks_stk::create(&h->stk, cfgs[0], h->stream, err);
        if (rc) {
            mks_destroy(h);
            return fail(rc, "%s", err.c_str());
        }
    }
    *out = h;
    return 0;
}

// Arm-chair stacking: the explicit-neighbour form of the lattice, expanded
// from the compact one after an initializer wrote it.
int stk_sync(mks_handle *h)
{
    if (!h->stk || !h->stk_dirty) return 0;
    const RepHost &r = h->reps[0];
    std::string err;
    int rc = mks_stk::from_compact(h->stk, h->d_st + r.st_off, r.NA, r.NB, r.NZ, r.pitch, err);
    if (rc) return fail(rc, "%s", err.c_str());
    h->stk_dirty = false;
    return 0;
}

int stk_unsupported(const char *what)
{
    return fail(MKS_ERR_UNSUPPORTED, "%s: not available with arm-chair stacking (PtransZig < 1)", what);
}

// tau = f / r*, r* the rate carrying the largest share of the total (the
// rule of mks_suggest_tau), from the explicit lists; dummies and isolated
// atoms do not count
int stk_suggest_tau(mks_handle *h, double f, double *tau)
{
    std::string err;
    std::vector<float> rate;
    int rc = mks_stk::event_rates(h->stk, rate, err);
    if (rc) return fail(rc, "%s", err.c_str());
    std::vector<std::pair<float, double>> share;
    std::sort(rate.begin(), rate.end());
    for (size_t i = 0; i < rate.size(); i++) {
        if (!(rate[i] > 1.e-6f)) continue;
        if (!share.empty() && share.back().first == rate[i]) share.back().second += rate[i];
        else share.push_back({rate[i], rate[i]});
    }
    if (share.empty()) return fail(MKS_ERR_ARG, "no event with a rate");
    auto best = std::max_element(share.begin(), share.end(),
                                 [](const std::pair<float, double> &a, const std::pair<float, double> &b) {
                                     return a.second < b.second;
                                 });
    *tau = f / (double)best->first;
    return 0;
}

// one window = one phase per colour + window end (a replica on the
// three-colour tiling has no tiles of colour 3)
int launch_window(mks_handle *h)
{
    for (int c = 0; c < 4; c++) {
        int nq = (int)h->color_list_h[c].size();
        if (!nq) continue;
        if (h->la_on)
            k_sl_phase<true><<<nq, 32, 0, h->stream>>>(h->d_reps, h->d_quads, h->d_clist[c], nq, h->d_st,
                                                       h->d_status, (uint32_t)c, h->d_la, h->d_score, h->d_tmaps);
        else if (h->any_cov)
            k_sl_phase<false, true><<<nq, 32, 0, h->stream>>>(h->d_reps, h->d_quads, h->d_clist[c], nq, h->d_st,
                                                              h->d_status, (uint32_t)c, h->d_la, h->d_score,
                                                              h->d_tmaps);
        else
            k_sl_phase<false><<<nq, 32, 0, h->stream>>>(h->d_reps, h->d_quads, h->d_clist[c], nq, h->d_st,
                                                        h->d_status, (uint32_t)c, h->d_la, h->d_score, h->d_tmaps);
        h->last_kernels++;
        h->last_phase_launches++;
    }
    k_window_end<<<(int)h->reps.size(), 256, 0, h->stream>>>(h->d_reps, h->d_quads, 1,
                                                             h->la_on ? h->d_la : nullptr);
    h->last_kernels++;
    CK(cudaGetLastError());
    return 0;
}

// Persistent schedule: one cooperative launch advances every tile through up
// to PERSIST_WINDOWS windows, then k_window_end advances the clocks and
// applies the exit conditions (checked per launch).
constexpr int PERSIST_WINDOWS = 256;
int run_persistent(mks_handle *h, int64_t max_windows)
{
    std::vector<RepDev> d;
    int nt = (int)h->quads_h.size();
    CK(cudaEventRecord(h->ev0, h->stream));
    int64_t done = 0;
    int launches = 0;
    while (done < max_windows) {
        int nw = (int)std::min<int64_t>(PERSIST_WINDOWS, max_windows - done);
        // LA: launches end on liquid-fraction refresh boundaries, as the
        // per-window schedule refreshes them
        if (h->la_on) nw = std::min<int64_t>(nw, LA_PHASE - (int64_t)(h->la_window % LA_PHASE));
        CK(cudaMemsetAsync(h->d_progress, 0xFF, sizeof(int) * (size_t)nt, h->stream));
        LADev *la = h->d_la;
        void *args[] = {&h->d_reps, &h->d_quads, &h->d_woff, &h->d_wtiles, &h->d_st, &h->d_status, &h->d_progress,
                        &nw, &la, &h->d_score, &h->d_tmaps, &h->spin_limit, &h->hold_tile};
        const void *fn = h->la_on ? (const void *)k_sl_persistent<true>
                         : h->any_cov ? (const void *)k_sl_persistent<false, true>
                                      : (const void *)k_sl_persistent<false>;
        CK(cudaLaunchCooperativeKernel(fn, dim3(h->coop_grid), dim3(32), args, 0, h->stream));
        k_window_end<<<(int)h->reps.size(), 256, 0, h->stream>>>(h->d_reps, h->d_quads, nw,
                                                                 h->la_on ? h->d_la : nullptr);
        h->la_window += nw;
        CK(cudaGetLastError());
        h->last_kernels += 2;
        h->last_phase_launches += 1;
        done += nw;
        launches++;
        if ((launches & 3) == 0 || done >= max_windows) {
            DevStatus s;
            int rc = read_status(h, s);
            if (rc) return rc;
            if (s.error) return fail(s.error, "device error %d in tile %d", s.error, s.err_quad);
            rc = download_reps(h, d);
            if (rc) return rc;
            bool any = false;
            for (auto &x : d) any |= x.active != 0;
            if (!any) break;
        }
    }
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaEventSynchronize(h->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    h->last_ms = ms;
    DevStatus s;
    int rc = read_status(h, s);
    if (rc) return rc;
    if (s.error) return fail(s.error, "device error %d in tile %d", s.error, s.err_quad);
    return 0;
}

int run_impl(mks_handle *h, const double *tau, int64_t max_windows, int64_t max_events, double max_time)
{
    NvtxRange nr("mks_run");
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    for (size_t i = 0; i < d.size(); i++) {
        if (!(tau[i] > 0.0)) return fail(MKS_ERR_ARG, "tau must be > 0");
        d[i].tau = tau[i];
        d[i].ev_max = max_events > 0 ? (long long)(d[i].events + (unsigned long long)max_events) : (long long)9e18;
        d[i].t_max = max_time > 0 ? max_time : 1e300;
        // "few MC particles" and "regrown" (LA) stops are final
        d[i].active = (d[i].stop_reason == 1 || d[i].stop_reason == 4) ? 0 : 1;
        if (d[i].active) d[i].stop_reason = 0;
    }
    rc = upload_reps(h, d);
    if (rc) return rc;
    h->last_kernels = 0;
    h->last_graphs = 0;
    h->last_phase_launches = 0;
    if (h->schedule == 1) return run_persistent(h, max_windows);
    // capture a block of windows once, replay it
    const int WPG = (int)std::max<int64_t>(1, std::min<int64_t>(8, max_windows));
    if (!h->graph_exec || h->graph_windows != WPG) {
        if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
        cudaGraph_t g;
        CK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
        int64_t k0 = h->last_kernels, p0 = h->last_phase_launches;
        for (int w = 0; w < WPG; w++) {
            int r2 = launch_window(h);
            if (r2) {
                cudaStreamEndCapture(h->stream, &g);
                return r2;
            }
        }
        h->last_kernels = k0;
        h->last_phase_launches = p0;
        CK(cudaStreamEndCapture(h->stream, &g));
        CK(cudaGraphInstantiate(&h->graph_exec, g, 0));
        cudaGraphDestroy(g);
        h->graph_windows = WPG;
    }
    int64_t kernels_per_graph = 0, phases_per_graph = 0;
    for (int c = 0; c < 4; c++)
        if (!h->color_list_h[c].empty()) phases_per_graph++;
    kernels_per_graph = (phases_per_graph + 1) * WPG;
    phases_per_graph *= WPG;
    CK(cudaEventRecord(h->ev0, h->stream));
    int64_t done = 0;
    while (done < max_windows) {
        CK(cudaGraphLaunch(h->graph_exec, h->stream));
        h->last_graphs++;
        h->la_window += WPG;
        h->last_kernels += kernels_per_graph;
        h->last_phase_launches += phases_per_graph;
        done += WPG;
        // poll the replica state every few blocks of windows
        if ((h->last_graphs & 7) == 0 || done >= max_windows) {
            DevStatus s;
            rc = read_status(h, s);
            if (rc) return rc;
            if (s.error) return fail(s.error, "device error %d in tile %d", s.error, s.err_quad);
            rc = download_reps(h, d);
            if (rc) return rc;
            bool any = false;
            for (auto &x : d) any |= x.active != 0;
            if (!any) break;
        }
    }
    CK(cudaEventRecord(h->ev1, h->stream));
    CK(cudaEventSynchronize(h->ev1));
    float ms = 0.f;
    CK(cudaEventElapsedTime(&ms, h->ev0, h->ev1));
    h->last_ms = ms;
    DevStatus s;
    rc = read_status(h, s);
    if (rc) return rc;
    if (s.error) return fail(s.error, "device error %d in tile %d", s.error, s.err_quad);
    return 0;
}

int obs_impl(mks_handle *h, int rep, mks_observables *o)
{
    NvtxRange nr("mks_observables");
    memset(o, 0, sizeof *o);
    unsigned long long *d_cnt = nullptr, *d_hist = nullptr;
    double *d_h = nullptr;
    CK(cudaMallocAsync(&d_cnt, sizeof(unsigned long long) * 8, h->stream));
    CK(cudaMallocAsync(&d_h, sizeof(double) * 2, h->stream));
    CK(cudaMallocAsync(&d_hist, sizeof(unsigned long long) * NCLASS, h->stream));
    CK(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long) * 8, h->stream));
    CK(cudaMemsetAsync(d_h, 0, sizeof(double) * 2, h->stream));
    CK(cudaMemsetAsync(d_hist, 0, sizeof(unsigned long long) * NCLASS, h->stream));
    const RepHost &r = h->reps[rep];
    int64_t ncol = (int64_t)r.NA * r.NB;
    int nslab = (r.NZ + OBS_ZSLAB - 1) / OBS_ZSLAB;
    int *d_top = nullptr;
    CK(cudaMallocAsync(&d_top, sizeof(int) * (size_t)ncol * nslab, h->stream));
    int64_t nthr = (int64_t)nslab * r.NB * (r.pitch / 16);
    k_observables<<<(int)std::min<int64_t>(152 * 8, (nthr + 255) / 256), 256, 0, h->stream>>>(h->d_reps, rep, h->d_st,
                                                                                              d_cnt, d_top);
    k_observables_heights<<<(int)std::min<int64_t>(152 * 4, (ncol + 255) / 256), 256, 0, h->stream>>>(
        d_top, ncol, nslab, d_cnt, d_h);
    class_hist(h, rep, rep + 1, d_hist);
    CK(cudaGetLastError());
    unsigned long long cnt[8], hist[NCLASS];
    double hs[2];
    CK(cudaMemcpyAsync(cnt, d_cnt, sizeof cnt, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(hs, d_h, sizeof hs, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(hist, d_hist, sizeof hist, cudaMemcpyDeviceToHost, h->stream));
    cudaFreeAsync(d_cnt, h->stream);
    cudaFreeAsync(d_h, h->stream);
    cudaFreeAsync(d_hist, h->stream);
    cudaFreeAsync(d_top, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    o->events = (int64_t)d[rep].events;
    o->time = d[rep].T0;
    o->atoms = (int64_t)cnt[0];
    o->undercoord = (int64_t)cnt[1];
    o->voids = (int64_t)cnt[2];
    o->species[0] = (int64_t)cnt[3];
    o->species[1] = (int64_t)cnt[4];
    o->species[2] = (int64_t)cnt[5];
    if (r.cfg.ncov) {              // the species-3 slot counted covered sites
        o->covered = o->species[2];
        o->species[2] = 0;
    }
    double ncols = (double)cnt[6];
    if (ncols > 0) {
        o->mean_height = hs[0] / ncols;
        double var = hs[1] / ncols - o->mean_height * o->mean_height;
        o->rms_roughness = var > 0 ? sqrt(var) : 0.0;
    }
    double rt = 0.0;
    int64_t mc = 0;
    for (int c = 1; c < NCLASS; c++) {
        mc += (int64_t)hist[c];
        if (c != CLS_ISO) rt += (double)hist[c] * (double)d[rep].rate[c];
    }
    rt += (double)hist[CLS_ISO] * 1.0e5 * rt;
    o->mc_sites = mc;
    o->total_rate = rt;
    o->nonepitaxial = 0;
    return 0;
}

}  // namespace

// ================================================================ C ABI
extern "C" {

const char *mks_version(void) { return "mulskips_gb300 0.1 (sm_103a)"; }

int mks_last_error(char *buf, int32_t len)
{
    if (!buf || len <= 0) return MKS_ERR_ARG;
    snprintf(buf, (size_t)len, "%s", g_err.c_str());
    return 0;
}

int mks_create(const mks_config *cfg, mks_handle **out) { return create_impl(cfg, 1, out); }
int mks_batch_create(const mks_config *cfgs, int32_t n, mks_handle **out) { return create_impl(cfgs, n, out); }
int32_t mks_batch_size(mks_handle *h) { return h ? (int32_t)h->reps.size() : 0; }

void mks_destroy(mks_handle *h)
{
    if (!h) return;
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    if (h->stream) cudaStreamSynchronize(h->stream);
    mks_stk::destroy(h->stk);
    cudaFree(h->d_st);
    cudaFree(h->d_reps);
    cudaFree(h->d_quads);
    cudaFree(h->d_status);
    cudaFree(h->d_progress);
    cudaFree(h->d_woff);
    cudaFree(h->d_wtiles);
    cudaFree(h->d_tmaps);
    cudaFree(h->d_st2);
    cudaFree(h->d_tmaps2);
    if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
    if (h->ev_copy) cudaEventDestroy(h->ev_copy);
    if (h->ev_swap) cudaEventDestroy(h->ev_swap);
    cudaFree(h->d_tfield);
    cudaFree(h->d_tlayer);
    cudaFree(h->d_la);
    if (h->d_lr) cudaFree(h->d_lr);
    if (h->d_lr_acc) cudaFree(h->d_lr_acc);
    cudaFree(h->d_score);
    for (int c = 0; c < 4; c++) cudaFree(h->d_clist[c]);
    if (h->ev0) cudaEventDestroy(h->ev0);
    if (h->ev1) cudaEventDestroy(h->ev1);
    if (h->stream) cudaStreamDestroy(h->stream);
    delete h;
}

int mks_batch_set_rates(mks_handle *h, const double *ptransE, const double *ptransD)
{
    if (!h || !ptransE || !ptransD) return fail(MKS_ERR_ARG, "bad arguments");
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    for (size_t i = 0; i < h->reps.size(); i++) {
        const double *pD = ptransD + i * 9;
        if (h->reps[i].cfg.ncov && (pD[6] != 0.0 || pD[7] != 0.0 || pD[8] != 0.0))
            return fail(MKS_ERR_UNSUPPORTED, "replica %zu: deposition of a third species with a coverage species", i);
        memcpy(h->reps[i].ptransE, ptransE + i * 3 * 4096, sizeof(double) * 3 * 4096);
        memcpy(h->reps[i].ptransD, pD, sizeof(double) * 9);
        h->reps[i].rates_set = true;
        rate_tables(h->reps[i], d[i]);
    }
    return upload_reps(h, d);
}

int mks_set_rates(mks_handle *h, const double *ptransE, const double *ptransD)
{
    if (!h || h->reps.size() != 1) return fail(MKS_ERR_ARG, "mks_set_rates needs a single-replica handle");
    int rc = mks_batch_set_rates(h, ptransE, ptransD);
    if (rc || !h->stk) return rc;
    std::string err;
    rc = mks_stk::set_rates(h->stk, ptransE, ptransD, err);
    return rc ? fail(rc, "%s", err.c_str()) : 0;
}

int mks_batch_set_coverage_rates(mks_handle *h, const double *ptransAbs, const double *ptransDes)
{
    if (!h || !ptransAbs || !ptransDes) return fail(MKS_ERR_ARG, "bad arguments");
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    for (size_t i = 0; i < h->reps.size(); i++) {
        RepHost &r = h->reps[i];
        if (!r.cfg.ncov) return fail(MKS_ERR_ARG, "replica %zu has no coverage species (NCov = 0)", i);
        for (int k = 0; k < 9; k++) {
            double a = ptransAbs[i * 9 + k], b = ptransDes[i * 9 + k];
            if (!(a >= 0.0) || !(b >= 0.0)) return fail(MKS_ERR_ARG, "negative or NaN coverage rate");
            if (k >= 3 * r.cfg.ncov && (a != 0.0 || b != 0.0))
                return fail(MKS_ERR_ARG, "replica %zu: rates for coverage species %d of NCov = %d", i, k / 3 + 1,
                            r.cfg.ncov);
        }
        memcpy(r.ptransAbs, ptransAbs + i * 9, sizeof(double) * 9);
        memcpy(r.ptransDes, ptransDes + i * 9, sizeof(double) * 9);
        rate_tables(r, d[i]);
    }
    return upload_reps(h, d);
}

int mks_set_coverage_rates(mks_handle *h, const double *ptransAbs, const double *ptransDes)
{
    if (!h || h->reps.size() != 1) return fail(MKS_ERR_ARG, "mks_set_coverage_rates needs a single-replica handle");
    return mks_batch_set_coverage_rates(h, ptransAbs, ptransDes);
}

int mks_batch_init_flat(mks_handle *h, char kind, const int32_t *len1)
{
    if (!h || !len1 || (kind != 'S' && kind != 'C')) return fail(MKS_ERR_ARG, "bad arguments");
    for (size_t i = 0; i < h->reps.size(); i++) {
        const RepHost &r = h->reps[i];
        int l1 = len1[i] - len1[i] % 24;
        if (l1 < 24 || l1 + 3 > r.cfg.lenz - 7) return fail(MKS_ERR_ARG, "Len1 %d outside the box", len1[i]);
        if (kind == 'C' && r.cfg.ncrystal < 2) return fail(MKS_ERR_ARG, "SiC needs NCrystal=2");
        int64_t n = (int64_t)r.NZ * r.NB * r.pitch;
        int blocks = (int)std::min<int64_t>(4096, (n + 255) / 256);
        k_init_flat<<<blocks, 256, 0, h->stream>>>(h->d_st + r.st_off, r.NA, r.NB, r.NZ, r.pitch, r.cfg.lenz, l1,
                                                   kind == 'C');
    }
    CK(cudaGetLastError());
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    for (auto &x : d) {
        x.T0 = 0.0;
        x.events = 0;
        x.window = 0;
        x.active = 1;
        x.stop_reason = 0;
    }
    rc = upload_reps(h, d);
    if (rc) return rc;
    return rescan(h);
}

int mks_init_flat(mks_handle *h, char kind, int32_t len1) { return mks_batch_init_flat(h, kind, &len1); }

int mks_batch_init_alloy(mks_handle *h, const int32_t *len1, const double *x, uint64_t seed)
{
    if (!h || !len1 || !x) return fail(MKS_ERR_ARG, "bad arguments");
    int rc = mks_batch_init_flat(h, 'S', len1);
    if (rc) return rc;
    for (size_t i = 0; i < h->reps.size(); i++) {
        const RepHost &r = h->reps[i];
        if (x[i] <= 0.0) continue;
        if (r.cfg.ncrystal < 2) return fail(MKS_ERR_ARG, "an alloy needs NCrystal >= 2");
        int l1 = len1[i] - len1[i] % 24;
        int64_t n = (int64_t)r.NZ * r.NB * r.pitch;
        int blocks = (int)std::min<int64_t>(4096, (n + 255) / 256);
        k_init_flat<<<blocks, 256, 0, h->stream>>>(h->d_st + r.st_off, r.NA, r.NB, r.NZ, r.pitch, r.cfg.lenz, l1, 0,
                                                   (float)x[i], seed + 0x9E3779B97F4A7C15ull * i);
    }
    CK(cudaGetLastError());
    return rescan(h);
}

int mks_batch_set_la(mks_handle *h, const mks_la_params *p, const double *dptransE, const double *dptransD)
{
    if (!h || !p) return fail(MKS_ERR_ARG, "bad arguments");
    size_t n = h->reps.size();
    std::vector<LADev> la(n);
    for (size_t i = 0; i < n; i++) {
        const RepHost &r = h->reps[i];
        if (r.cfg.ncov) return fail(MKS_ERR_UNSUPPORTED, "LA mode needs NCov = 0 (main.f:118-123)");
        LADev &A = la[i];
        memset(&A, 0, sizeof A);
        A.on = 1;
        A.score_on = p[i].score ? 1 : 0;
        for (int s = 0; s < 3; s++) {
            A.P0[s] = p[i].P0[s];
            A.Tm[s] = p[i].Tm[s] > 0 ? p[i].Tm[s] : 1.f;
            A.Tflex[s] = p[i].Tflex[s];
            A.sigma[s] = p[i].sigma[s] > 0 ? p[i].sigma[s] : 1.f;
        }
        A.Tb = p[i].Tb;
        A.Ta = p[i].Ta;
        A.t0 = p[i].t0;
        A.w = p[i].w > 0 ? p[i].w : 1.f;
        A.L = p[i].L_nm > 0 ? p[i].L_nm : 1e30f;
        A.zsurf = p[i].zsurf;
        A.sf = (float)r.cfg.sf;
        A.liquid_weighting = p[i].liquid_weighting ? 1 : 0;
        A.swap_species = A.liquid_weighting && r.cfg.ncrystal == 2 && r.cfg.list_crystal[0] == 14 &&
                         r.cfg.list_crystal[1] == 32;
        if (r.t_layer_off >= 0) {
            A.tfield = h->d_tfield + r.st_off;
            A.tlayer = h->d_tlayer + r.t_layer_off;
            A.tNA = r.NA;
            A.tNB = r.NB;
            A.tpitch = r.pitch;
        }
        // barriers: the PTransE / PTransD tables given to mks_batch_set_rates (eV)
        for (int sp = 1; sp <= 3; sp++)
            for (int n1 = 0; n1 <= 3; n1++)
                for (int n2 = 0; n2 <= 3; n2++)
                    for (int n3 = 0; n3 <= 3; n3++) {
                        int t = n1 + n2 + n3;
                        if (t < 1 || t > 3) continue;
                        int c = CLS_OCC0 + (sp - 1) * NCENSUS + census_index(n1, n2, n3);
                        size_t k = (size_t)(sp - 1) * 4096 + n1 * 1024 + n2 * 256 + n3 * 64;
                        A.E[c] = (float)r.ptransE[k];
                        if (dptransE)
                            for (int j = 0; j < 4; j++) A.dE[c][j] = (float)dptransE[(i * 3 * 4096 + k) * 4 + j];
                    }
        for (int sp = 0; sp < 3; sp++)
            for (int co = 0; co < 3; co++) {
                A.Edep[sp][co] = (float)r.ptransD[sp * 3 + co];
                if (dptransD)
                    for (int j = 0; j < 4; j++) A.dEdep[sp][co][j] = (float)dptransD[(i * 9 + sp * 3 + co) * 4 + j];
            }
    }
    // crystal atoms now: nothing is liquid yet (InitCountCrystal = CountCrystal);
    // the MS law has no liquid fraction (it is 1 for every species)
    {
        int64_t umax = 0;
        for (const RepHost &r : h->reps) umax = std::max<int64_t>(umax, (int64_t)r.NZ * r.NB * (r.pitch / 16));
        unsigned long long *d_cnt = nullptr;
        CK(cudaMallocAsync(&d_cnt, sizeof(unsigned long long) * 3 * n, h->stream));
        CK(cudaMemsetAsync(d_cnt, 0, sizeof(unsigned long long) * 3 * n, h->stream));
        for (size_t r0 = 0; r0 < n; r0 += 65535) {
            dim3 grid((unsigned)std::max<int64_t>(1, std::min<int64_t>(1024, umax / 4096)),
                      (unsigned)std::min<size_t>(65535, n - r0));
            k_species_counts<<<grid, 256, 0, h->stream>>>(h->d_reps, (int)r0, h->d_st, d_cnt);
        }
        CK(cudaGetLastError());
        std::vector<unsigned long long> cnt(3 * n);
        CK(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(unsigned long long) * 3 * n, cudaMemcpyDeviceToHost, h->stream));
        cudaFreeAsync(d_cnt, h->stream);
        CK(cudaStreamSynchronize(h->stream));
        for (size_t i = 0; i < n; i++)
            for (int s = 0; s < 3; s++) {
                la[i].init_cnt[s] = la[i].cnt[s] = (long long)cnt[3 * i + s];
                if (!la[i].liquid_weighting) la[i].xliq[s] = 1.f;
            }
    }
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    h->la_window = d.empty() ? 0 : d[0].window;
    // a captured window graph holds the plain kernels: capture again
    if (h->graph_exec) {
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
    }
    CK(cudaMemcpyAsync(h->d_la, la.data(), sizeof(LADev) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->d_score, 0, sizeof(double) * 4 * n, h->stream));
    if (h->d_lr_acc) CK(cudaMemsetAsync(h->d_lr_acc, 0, sizeof(double) * 4 * n, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->la_on = 1;
    return 0;
}

int mks_batch_set_tabulated(mks_handle *h, int32_t ntemp, const int32_t *temps, const double *ptransE,
                            const double *ptransD)
{
    if (!h || !temps || !ptransE || !ptransD) return fail(MKS_ERR_ARG, "bad arguments");
    if (ntemp < 1 || ntemp > LA_NTAB) return fail(MKS_ERR_ARG, "ntemp %d outside 1..%d", ntemp, LA_NTAB);
    size_t n = h->reps.size();
    std::vector<LADev> la(n);
    for (size_t i = 0; i < n; i++) {
        const RepHost &r = h->reps[i];
        if (r.cfg.ncov) return fail(MKS_ERR_UNSUPPORTED, "tabulated rates with a coverage species");
        if (r.t_layer_off < 0) return fail(MKS_ERR_ARG, "replica %zu: load its temperature field first", i);
        LADev &A = la[i];
        memset(&A, 0, sizeof A);
        A.on = 1;
        A.sf = (float)r.cfg.sf;
        A.tfield = h->d_tfield + r.st_off;
        A.tlayer = h->d_tlayer + r.t_layer_off;
        A.tNA = r.NA;
        A.tNB = r.NB;
        A.tpitch = r.pitch;
        A.ntab = ntemp;
        for (int s = 0; s < 3; s++) {
            A.xliq[s] = 1.f;
            A.Tm[s] = A.sigma[s] = A.w = A.L = 1.f;
        }
        for (int k = 0; k < ntemp; k++) {
            A.tabT[k] = (float)temps[i * ntemp + k];
            if (k && !(A.tabT[k] > A.tabT[k - 1]))
                return fail(MKS_ERR_ARG, "replica %zu: table temperatures must increase", i);
            RepHost row = r;                   // the class mapping of rate_tables on row k
            memcpy(row.ptransE, ptransE + ((size_t)i * ntemp + k) * 3 * 4096, sizeof row.ptransE);
            memcpy(row.ptransD, ptransD + ((size_t)i * ntemp + k) * 9, sizeof row.ptransD);
            RepDev d;
            memset(&d, 0, sizeof d);
            rate_tables(row, d);
            for (int c = 0; c < 64; c++) A.tabE[k][c] = (c >= CLS_OCC0 && c < CLS_C1I) ? d.rate[c] : 0.f;
            for (int sp = 0; sp < 3; sp++)
                for (int co = 0; co < 3; co++) A.tabD[k][sp][co] = (float)row.ptransD[sp * 3 + co];
        }
        // the per-tile bound takes the rates at the hottest staged layer
        for (int k = 1; k < ntemp; k++) {
            for (int c = CLS_OCC0; c < CLS_C1I; c++)
                if (A.tabE[k][c] < A.tabE[k - 1][c])
                    return fail(MKS_ERR_UNSUPPORTED, "replica %zu: tabulated rate of class %d decreases with T", i, c);
            for (int co = 0; co < 3; co++) {
                float a = 0.f, b = 0.f;
                for (int sp = 0; sp < 3; sp++) {
                    a += A.tabD[k - 1][sp][co];
                    b += A.tabD[k][sp][co];
                }
                if (b < a) return fail(MKS_ERR_UNSUPPORTED, "replica %zu: tabulated deposition decreases with T", i);
            }
        }
    }
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    h->la_window = d.empty() ? 0 : d[0].window;
    if (h->graph_exec) {
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
    }
    CK(cudaMemcpyAsync(h->d_la, la.data(), sizeof(LADev) * n, cudaMemcpyHostToDevice, h->stream));
    CK(cudaMemsetAsync(h->d_score, 0, sizeof(double) * 4 * n, h->stream));
    if (h->d_lr_acc) CK(cudaMemsetAsync(h->d_lr_acc, 0, sizeof(double) * 4 * n, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    h->la_on = 1;
    return 0;
}

int mks_batch_lr_grad(mks_handle *h, const double *f, int32_t use_baseline, double *grad, double *se)
{
    if (!h || !f || !grad) return fail(MKS_ERR_ARG, "bad arguments");
    if (!h->la_on) return fail(MKS_ERR_ARG, "LA mode is not set (mks_batch_set_la)");
    int n = (int)h->reps.size();
    if (!h->d_lr) CK(cudaMalloc(&h->d_lr, sizeof(double) * (size_t)(n + 8)));
    CK(cudaMemcpyAsync(h->d_lr, f, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    k_lr_grad<<<1, 256, 0, h->stream>>>(h->d_score, h->d_lr, n, use_baseline ? 1 : 0, h->d_lr + n);
    CK(cudaGetLastError());
    double out[8];
    CK(cudaMemcpyAsync(out, h->d_lr + n, sizeof out, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int j = 0; j < 4; j++) {
        grad[j] = out[j];
        if (se) se[j] = out[4 + j];
    }
    return 0;
}

int mks_batch_lr_accumulate(mks_handle *h, const double *df)
{
    if (!h || !df) return fail(MKS_ERR_ARG, "bad arguments");
    if (!h->la_on) return fail(MKS_ERR_ARG, "LA mode is not set (mks_batch_set_la)");
    int n = (int)h->reps.size();
    if (!h->d_lr) CK(cudaMalloc(&h->d_lr, sizeof(double) * (size_t)(n + 8)));
    if (!h->d_lr_acc) {
        CK(cudaMalloc(&h->d_lr_acc, sizeof(double) * (size_t)(5 * n + 8)));
        CK(cudaMemsetAsync(h->d_lr_acc, 0, sizeof(double) * 4 * (size_t)n, h->stream));
    }
    CK(cudaMemcpyAsync(h->d_lr, df, sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    k_lr_step<<<1, 256, 0, h->stream>>>(h->d_score, h->d_lr, n, h->d_lr_acc);
    CK(cudaGetLastError());
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int mks_batch_lr_result(mks_handle *h, int32_t reset, double *grad, double *se)
{
    if (!h || !grad) return fail(MKS_ERR_ARG, "bad arguments");
    if (!h->d_lr_acc) return fail(MKS_ERR_ARG, "no mks_batch_lr_accumulate since the last reset");
    int n = (int)h->reps.size();
    // the mean over replicas of the causal sums and its standard error: the
    // reduction of k_lr_grad with f = 1 and no baseline
    std::vector<double> ones((size_t)n, 1.0);
    double *d_one = h->d_lr_acc + 4 * (size_t)n;
    CK(cudaMemcpyAsync(d_one, ones.data(), sizeof(double) * n, cudaMemcpyHostToDevice, h->stream));
    k_lr_grad<<<1, 256, 0, h->stream>>>(h->d_lr_acc, d_one, n, 0, d_one + n);
    CK(cudaGetLastError());
    double out[8];
    CK(cudaMemcpyAsync(out, d_one + n, sizeof out, cudaMemcpyDeviceToHost, h->stream));
    if (reset) CK(cudaMemsetAsync(h->d_lr_acc, 0, sizeof(double) * 4 * (size_t)n, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (int j = 0; j < 4; j++) {
        grad[j] = out[j];
        if (se) se[j] = out[4 + j];
    }
    return 0;
}

int mks_batch_la_counts(mks_handle *h, int64_t *crystal, double *xliq)
{
    if (!h || !crystal) return fail(MKS_ERR_ARG, "bad arguments");
    if (!h->la_on) return fail(MKS_ERR_ARG, "LA mode is not set (mks_batch_set_la)");
    size_t n = h->reps.size();
    // the counters lead each replica's LADev: copy that head only
    struct Head {
        long long init_cnt[3], cnt[3];
        float xliq[3];
    };
    static_assert(offsetof(LADev, init_cnt) == 0 && offsetof(LADev, cnt) == offsetof(Head, cnt) &&
                      offsetof(LADev, xliq) == offsetof(Head, xliq),
                  "LADev starts with its counters");
    std::vector<Head> hd(n);
    CK(cudaMemcpy2DAsync(hd.data(), sizeof(Head), h->d_la, sizeof(LADev), offsetof(Head, xliq) + sizeof(float) * 3, n,
                         cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < n; i++)
        for (int s = 0; s < 3; s++) {
            crystal[3 * i + s] = hd[i].cnt[s];
            if (xliq) xliq[3 * i + s] = hd[i].xliq[s];
        }
    return 0;
}

int mks_batch_get_score(mks_handle *h, double *score, int32_t reset)
{
    if (!h || !score) return fail(MKS_ERR_ARG, "bad arguments");
    size_t n = h->reps.size();
    CK(cudaMemcpyAsync(score, h->d_score, sizeof(double) * 4 * n, cudaMemcpyDeviceToHost, h->stream));
    if (reset) CK(cudaMemsetAsync(h->d_score, 0, sizeof(double) * 4 * n, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int64_t mks_state_size(mks_handle *h)
{
    if (!h || h->reps.empty()) return 0;
    const RepHost &r = h->reps[0];
    return (int64_t)r.NZ * r.NB * r.NA;
}

int mks_get_state(mks_handle *h, uint8_t *out, int64_t n)
{
    if (!h || !out || n < mks_state_size(h)) return fail(MKS_ERR_ARG, "bad arguments");
    if (h->stk && !h->stk_dirty) return stk_unsupported("mks_get_state (see mks_get_lattice)");
    const RepHost &r = h->reps[0];
    if (r.NA == r.pitch)
        CK(cudaMemcpyAsync(out, h->d_st + r.st_off, (size_t)mks_state_size(h), cudaMemcpyDeviceToHost, h->stream));
    else
        CK(cudaMemcpy2DAsync(out, r.NA, h->d_st + r.st_off, r.pitch, r.NA, (size_t)r.NZ * r.NB,
                             cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int mks_batch_get_state(mks_handle *h, int32_t rep, uint8_t *out, int64_t n)
{
    if (!h || !out || rep < 0 || rep >= (int)h->reps.size()) return fail(MKS_ERR_ARG, "bad arguments");
    const RepHost &r = h->reps[rep];
    const int64_t need = (int64_t)r.NZ * r.NB * r.NA;
    if (n < need) return fail(MKS_ERR_ARG, "buffer of %lld bytes, %lld needed", (long long)n, (long long)need);
    CK(cudaMemcpy2DAsync(out, r.NA, h->d_st + r.st_off, r.pitch, r.NA, (size_t)r.NZ * r.NB, cudaMemcpyDeviceToHost,
                         h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int mks_prefetch_state(mks_handle *h, const uint8_t *in, int64_t n)
{
    if (!h || !in || n < mks_state_size(h) || h->reps.size() != 1) return fail(MKS_ERR_ARG, "bad arguments");
    const RepHost &r = h->reps[0];
    if (!h->d_st2) {
        CK(cudaMalloc(&h->d_st2, (size_t)h->st_bytes));
        CK(cudaMemset(h->d_st2, 0, (size_t)h->st_bytes));
        CK(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
        CK(cudaEventCreateWithFlags(&h->ev_copy, cudaEventDisableTiming));
        CK(cudaEventCreateWithFlags(&h->ev_swap, cudaEventDisableTiming));
        int rc = make_tensor_maps(h, h->d_st2, &h->d_tmaps2);
        if (rc) return rc;
    }
    // the buffer may still be read by work queued before the last swap
    CK(cudaStreamWaitEvent(h->copy_stream, h->ev_swap, 0));
    if (r.NA == r.pitch)
        CK(cudaMemcpyAsync(h->d_st2 + r.st_off, in, (size_t)mks_state_size(h), cudaMemcpyHostToDevice,
                           h->copy_stream));
    else
        CK(cudaMemcpy2DAsync(h->d_st2 + r.st_off, r.pitch, in, r.NA, r.NA, (size_t)r.NZ * r.NB, cudaMemcpyHostToDevice,
                             h->copy_stream));
    CK(cudaEventRecord(h->ev_copy, h->copy_stream));
    h->prefetched = true;
    return 0;
}

int mks_swap_state(mks_handle *h)
{
    if (!h || !h->prefetched) return fail(MKS_ERR_ARG, "no state prefetched (mks_prefetch_state)");
    CK(cudaStreamWaitEvent(h->stream, h->ev_copy, 0));
    std::swap(h->d_st, h->d_st2);
    std::swap(h->d_tmaps, h->d_tmaps2);
    if (h->graph_exec) {                   // captured windows hold the old lattice pointer
        cudaGraphExecDestroy(h->graph_exec);
        h->graph_exec = nullptr;
    }
    h->prefetched = false;
    CK(cudaEventRecord(h->ev_swap, h->stream));
    return rescan(h);
}

int mks_set_state(mks_handle *h, const uint8_t *in, int64_t n)
{
    if (!h || !in || n < mks_state_size(h) || h->reps.size() != 1) return fail(MKS_ERR_ARG, "bad arguments");
    const RepHost &r = h->reps[0];
    if (r.NA == r.pitch)
        CK(cudaMemcpyAsync(h->d_st + r.st_off, in, (size_t)mks_state_size(h), cudaMemcpyHostToDevice, h->stream));
    else
        CK(cudaMemcpy2DAsync(h->d_st + r.st_off, r.pitch, in, r.NA, r.NA, (size_t)r.NZ * r.NB,
                             cudaMemcpyHostToDevice, h->stream));
    return rescan(h);
}

int mks_load_lists(mks_handle *h, const int32_t *lattcoo, int64_t n, const int32_t *xyz, const int32_t *nn,
                   const int32_t *event, const float *rate)
{
    if (!h || !lattcoo || n < 0 || (n && (!xyz || !nn)) || (!event) != (!rate)) return fail(MKS_ERR_ARG, "bad arguments");
    if (!h->stk) return fail(MKS_ERR_ARG, "mks_load_lists needs a handle with PtransZig < 1");
    std::string err;
    int rc = mks_stk::load_lists(h->stk, lattcoo, n, xyz, nn, event, rate, err);
    if (rc) return fail(rc, "%s", err.c_str());
    h->stk_dirty = false;
    return 0;
}

int mks_get_lists(mks_handle *h, int64_t cap, int32_t *xyz, int32_t *nn, int32_t *kind, int32_t *event, float *rate,
                  int64_t *n)
{
    if (!h || !n) return fail(MKS_ERR_ARG, "bad arguments");
    if (!h->stk) return fail(MKS_ERR_ARG, "mks_get_lists needs a handle with PtransZig < 1");
    int rc = stk_sync(h);
    if (rc) return rc;
    std::string err;
    rc = mks_stk::get_lists(h->stk, cap, xyz, nn, kind, event, rate, n, err);
    return rc ? fail(rc, "%s", err.c_str()) : 0;
}

int mks_get_lattice(mks_handle *h, int32_t *lc)
{
    if (!h || !lc) return fail(MKS_ERR_ARG, "bad arguments");
    if (h->stk && !h->stk_dirty) {
        std::string err;
        int rc = mks_stk::get_lattice(h->stk, lc, err);
        return rc ? fail(rc, "%s", err.c_str()) : 0;
    }
    const RepHost &r = h->reps[0];
    std::vector<uint8_t> st((size_t)mks_state_size(h));
    int rc = mks_get_state(h, st.data(), (int64_t)st.size());
    if (rc) return rc;
    int lx = r.cfg.lenx, ly = r.cfg.leny, lz = r.cfg.lenz;
    memset(lc, 0, sizeof(int32_t) * (size_t)lx * ly * (lz + 1));
    // wall planes of SetSi cover every grid point (SetSi.f:38-46,212-220):
    // a wall layer z1 stands for grid planes 3*z1 .. 3*z1+2
    for (int z1 = 0; z1 < r.NZ; z1++) {
        if (st[(size_t)z1 * r.NB * r.NA + (size_t)((z1 >> 1) & 1)] != WALL) continue;
        for (int zz = 3 * z1; zz < 3 * z1 + 3 && zz <= lz; zz++)
            for (size_t k = 0; k < (size_t)lx * ly; k++) lc[(size_t)lx * ly * zz + k] = (1 << 23) | 113;
    }
    for (int z1 = 0; z1 < r.NZ; z1++)
        for (int b = 0; b < r.NB; b++)
            for (int a = 0; a < r.NA; a++) {
                uint8_t s = st[((size_t)z1 * r.NB + b) * r.NA + a];
                if (((a + b + (z1 >> 1)) & 1) || s == 0) continue;
                int x = 3 * (2 * a + (z1 & 1)), y = 3 * (2 * b + (z1 & 1)), z = 3 * z1;
                if (z > lz) continue;
                int32_t v;
                if (s == WALL) continue;
                int sp = sp_of(s), co = co_of(s);
                if (r.cfg.ncov && sp == COVSP)      // covered empty site: CovInd = ListCov(i), absorption.f:34-36
                    v = (co << 24) | r.cfg.list_cov[(s & COV2) ? 1 : 0];
                else
                    v = (co << 24) | (sp ? (1 << 23) : 0) | (sp << 27);
                lc[(size_t)x + (size_t)lx * ((size_t)y + (size_t)ly * z)] = v;
            }
    return 0;
}

int upload_compact(mks_handle *h, int rep, std::vector<uint8_t> &st, bool ini = true);

// A host-built lattice (mks_shapes::Grid, rows of NA bytes) into the padded
// rows of replica rep, then upload_compact (ini: the initializer rates its
// sites with Get_Prob_Ini).
int upload_grid(mks_handle *h, int rep, const mks_shapes::Grid &g, bool ini = true)
{
    const RepHost &r = h->reps[rep];
    std::vector<uint8_t> st((size_t)r.NZ * r.NB * r.pitch, 0);
    for (int z1 = 0; z1 < r.NZ; z1++)
        for (int b = 0; b < r.NB; b++)
            memcpy(&st[((size_t)z1 * r.NB + b) * r.pitch], &g.st[((size_t)z1 * r.NB + b) * r.NA], (size_t)r.NA);
    return upload_compact(h, rep, st, ini);
}

int load_lattice_impl(mks_handle *h, int rep, const int32_t *lc)
{
    const RepHost &r = h->reps[rep];
    int lx = r.cfg.lenx, ly = r.cfg.leny;
    std::vector<uint8_t> st((size_t)r.NZ * r.NB * r.pitch, 0);
    auto at = [&](int a, int b, int z) -> uint8_t & {
        a = (a % r.NA + r.NA) % r.NA;
        b = (b % r.NB + r.NB) % r.NB;
        return st[((size_t)z * r.NB + b) * r.pitch + a];
    };
    for (int z1 = 0; z1 < r.NZ; z1++)
        for (int b = 0; b < r.NB; b++)
            for (int a = 0; a < r.NA; a++) {
                if ((a + b + (z1 >> 1)) & 1) continue;
                int x = 3 * (2 * a + (z1 & 1)), y = 3 * (2 * b + (z1 & 1)), z = 3 * z1;
                int32_t v = lc[(size_t)x + (size_t)lx * ((size_t)y + (size_t)ly * z)];
                if ((v & 255) == 113) {
                    at(a, b, z1) = WALL;
                    continue;
                }
                int occ = (v >> 23) & 1, co = (v >> 24) & 7, sp = (v >> 27) & 7;
                if ((v & 255) != 0) {
                    const int ci = (v & 255) == r.cfg.list_cov[0] ? 1 : ((r.cfg.ncov == 2 && (v & 255) == r.cfg.list_cov[1]) ? 2 : 0);
                    if (!r.cfg.ncov || !ci) return fail(MKS_ERR_UNSUPPORTED, "coverage index %d in LattCoo", v & 255);
                    if (occ || sp || co < 1 || co > 4) return fail(MKS_ERR_INVARIANT, "bad covered LattCoo word %d", v);
                    at(a, b, z1) = (uint8_t)(mk(COVSP, co, 0, 0) | (ci == 2 ? COV2 : 0));
                    continue;
                }
                if (sp > (r.cfg.ncov ? 2 : 3) || (occ && !sp) || (!occ && sp))
                    return fail(MKS_ERR_INVARIANT, "bad LattCoo word %d", v);
                at(a, b, z1) = mk(sp, co, 0, 0);
            }
    return upload_compact(h, rep, st);
}

// The first list entry and dummy flag of coor-1 sites, then the upload of the
// padded compact state st of replica rep and the event-site scan.  A lattice
// loaded as LattCoo is an initial lattice: its lists are rebuilt as SetCAD.f:
// 301-418 does, and its dummies take Get_Prob_Ini's rate (ini), as do those
// of every initializer but SetSiC3Cww(aperture).
int upload_compact(mks_handle *h, int rep, std::vector<uint8_t> &st, bool ini)
{
    const RepHost &r = h->reps[rep];
    auto at = [&](int a, int b, int z) -> uint8_t & {
        a = (a % r.NA + r.NA) % r.NA;
        b = (b % r.NB + r.NB) % r.NB;
        return st[((size_t)z * r.NB + b) * r.pitch + a];
    };
    // the first list entry of a coor-1 empty site is its one occupied
    // neighbour; its dummy flag follows that neighbour's coordination
    // (Get_Prob.f:156-184), as a rebuild from LattCoo gives (SetCAD.f:301-418)
    for (int z1 = 0; z1 < r.NZ; z1++)
        for (int b = 0; b < r.NB; b++)
            for (int a = 0; a < r.NA; a++) {
                if ((a + b + (z1 >> 1)) & 1) continue;
                uint8_t s = at(a, b, z1);
                const bool cov = r.cfg.ncov != 0;
                bool covered = is_cov(s, cov);
                if (s == WALL || (sp_of(s) && !covered) || co_of(s) != 1) continue;
                int found = -1;
                uint8_t ns = 0;
                for (int d = 0; d < 4; d++) {
                    int da, db, dz;
                    nb_off(z1 & 1, d, da, db, dz);
                    if (z1 + dz < 0 || z1 + dz >= r.NZ) continue;
                    uint8_t t = at(a + da, b + db, z1 + dz);
                    if (t != WALL && atom_sp(t, cov)) {
                        found = d;
                        ns = t;
                    }
                }
                if (found < 0) return fail(MKS_ERR_INVARIANT, "coor-1 site without neighbour");
                at(a, b, z1) = covered ? (uint8_t)(mk(COVSP, 1, found, 0) | (s & COV2)) : mk_c1(found, co_of(ns), ini);
            }
    CK(cudaMemcpyAsync(h->d_st + r.st_off, st.data(), st.size(), cudaMemcpyHostToDevice, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    return rescan(h);
}

int mks_load_lattice(mks_handle *h, const int32_t *lc)
{
    if (!h || !lc || h->reps.size() != 1) return fail(MKS_ERR_ARG, "bad arguments");
    return load_lattice_impl(h, 0, lc);
}

int mks_batch_load_lattice(mks_handle *h, int32_t rep, const int32_t *lc)
{
    if (!h || !lc || rep < 0 || rep >= (int)h->reps.size()) return fail(MKS_ERR_ARG, "bad arguments");
    return load_lattice_impl(h, rep, lc);
}

}  // extern "C"

namespace {

// The LA temperature field of replica rep from a per-grid-point source:
// T(x, y, z, previous) gives each diamond site's temperature.
template <class F>
int set_temperature_impl(mks_handle *h, int rep, F temp_of)
{
    if (!h->d_tfield) {
        int64_t nl = 0;
        for (RepHost &x : h->reps) nl += x.NZ;
        CK(cudaMalloc(&h->d_tfield, sizeof(uint16_t) * (size_t)h->st_bytes));
        CK(cudaMemset(h->d_tfield, 0, sizeof(uint16_t) * (size_t)h->st_bytes));
        CK(cudaMalloc(&h->d_tlayer, sizeof(float) * (size_t)nl));
        CK(cudaMemset(h->d_tlayer, 0, sizeof(float) * (size_t)nl));
        for (RepHost &x : h->reps) x.t_layer_off = -1;
    }
    RepHost &r = h->reps[rep];
    int64_t loff = 0;
    for (int i = 0; i < rep; i++) loff += h->reps[i].NZ;
    std::vector<uint16_t> t((size_t)r.NZ * r.NB * r.pitch, 0);
    CK(cudaStreamSynchronize(h->stream));
    CK(cudaMemcpy(t.data(), h->d_tfield + r.st_off, sizeof(uint16_t) * t.size(), cudaMemcpyDeviceToHost));
    std::vector<float> tl((size_t)r.NZ, 0.f);
    for (int z1 = 0; z1 < r.NZ; z1++)
        for (int b = 0; b < r.NB; b++)
            for (int a = 0; a < r.NA; a++) {
                if ((a + b + (z1 >> 1)) & 1) continue;
                int x = 3 * (2 * a + (z1 & 1)), y = 3 * (2 * b + (z1 & 1)), z = 3 * z1;
                uint16_t &v = t[((size_t)z1 * r.NB + b) * r.pitch + a];
                int T = z < r.cfg.lenz ? temp_of(x, y, z, (int)v) : (int)v;
                v = (uint16_t)T;
                tl[z1] = std::max(tl[z1], (float)T);
            }
    CK(cudaMemcpy(h->d_tfield + r.st_off, t.data(), sizeof(uint16_t) * t.size(), cudaMemcpyHostToDevice));
    CK(cudaMemcpy(h->d_tlayer + loff, tl.data(), sizeof(float) * tl.size(), cudaMemcpyHostToDevice));
    r.t_layer_off = loff;
    return 0;
}

// Phases of the LA coupling messages (LaserAnnealing main.f:796-817), one
// thread per grid point of the socket layout: index z + LenZ (x + LenX y).
__global__ void k_wall_layers(const RepDev *reps, int rep, const uint8_t *st_all, int *wall)
{
    const RepDev &R = reps[rep];
    const uint8_t *st = st_all + R.st_off;
    int64_t n = (int64_t)R.NZ * R.NB * R.NA;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int a = (int)(i % R.NA);
        int64_t r = i / R.NA;
        int b = (int)(r % R.NB), z1 = (int)(r / R.NB);
        if ((a + b + (z1 >> 1)) & 1) continue;
        if (st[((int64_t)z1 * R.NB + b) * R.pitch + a] != WALL) wall[z1] = 0;
    }
}

__global__ void k_phases(const RepDev *reps, int rep, const uint8_t *st_all, int lx, int ly, int lz,
                         const int *wall, int32_t *coo, int32_t *spc)
{
    const RepDev &R = reps[rep];
    const uint8_t *st = st_all + R.st_off;
    const bool cov = R.cov != 0;
    int64_t n = (int64_t)lz * lx * ly;
    for (int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; i < n; i += (int64_t)gridDim.x * blockDim.x) {
        int z = (int)(i % lz);
        int64_t r = i / lz;
        int x = (int)(r % lx), y = (int)(r / lx);
        int z1 = z / 3, c = 0, s = 0;
        bool site = false;
        if (x % 3 == 0 && y % 3 == 0 && z % 3 == 0) {
            int x1 = x / 3, y1 = y / 3;
            if ((x1 & 1) == (z1 & 1) && (y1 & 1) == (z1 & 1) && (((x1 >> 1) + (y1 >> 1) + (z1 >> 1)) & 1) == 0) {
                site = true;
                uint8_t v = st[((int64_t)z1 * R.NB + (y1 >> 1)) * R.pitch + (x1 >> 1)];
                int sp = atom_sp(v, cov);
                if (v == WALL) {
                    c = s = 10;
                } else if (sp) {
                    c = co_of(v);
                    s = sp;
                }
            }
        }
        if (!site && z1 < R.NZ && wall[z1]) c = s = 10;
        if (coo) coo[i] = c;
        if (spc) spc[i] = s;
    }
}

}  // namespace

extern "C" {

int mks_batch_load_temperature(mks_handle *h, int32_t rep, const int32_t *lc)
{
    if (!h || !lc || rep < 0 || rep >= (int)h->reps.size()) return fail(MKS_ERR_ARG, "bad arguments");
    const int lx = h->reps[rep].cfg.lenx, ly = h->reps[rep].cfg.leny;
    return set_temperature_impl(h, rep, [&](int x, int y, int z, int) {
        return (lc[(size_t)x + (size_t)lx * ((size_t)y + (size_t)ly * z)] >> 9) & 8191;   // PosT, LenT
    });
}

int mks_batch_set_field(mks_handle *h, int32_t rep, const int32_t *field)
{
    if (!h || !field || rep < 0 || rep >= (int)h->reps.size()) return fail(MKS_ERR_ARG, "bad arguments");
    const int lx = h->reps[rep].cfg.lenx, lz = h->reps[rep].cfg.lenz;
    for (size_t i = 0, n = (size_t)lz * lx * h->reps[rep].cfg.leny; i < n; i++)
        if (field[i] < 0 || field[i] > 8191) return fail(MKS_ERR_ARG, "temperature %d K outside the 13-bit field", field[i]);
    // SetT (LaserAnnealing initial/SetT.f:34-48): 10 marks a wall and keeps the site's temperature
    return set_temperature_impl(h, rep, [&](int x, int y, int z, int old) {
        int T = field[(size_t)z + (size_t)lz * ((size_t)x + (size_t)lx * y)];
        return T == 10 ? old : T;
    });
}

// InitSt E, SetSiCSF (main.f:267-272 passes Len1 and the vertex (Len2,
// Len3, Len1 - Len2)): built on the host (sicsf.h) as LattCoo and the
// reference's lists, loaded into the explicit-neighbour engine, which rates
// every entry from that state.  The fault's atoms lie off the diamond sites,
// which the compact lattice cannot hold.
static int init_sicsf(mks_handle *h, const int32_t *lens)
{
    if (!h->stk)
        return fail(MKS_ERR_UNSUPPORTED, "InitSt E (SetSiCSF) places atoms off the diamond sites: it needs the "
                                         "explicit-neighbour engine (PtransZig < 1 or mks_config.explicit_nn = 1)");
    const mks_config &c = h->reps[0].cfg;
    mks_sicsf::Result R;
    const int vsf[3] = {lens[1], lens[2], lens[0] - lens[1]};
    const std::string e = mks_sicsf::build(c.lenx, c.leny, c.lenz, lens[0], vsf, R);
    if (!e.empty()) return fail(MKS_ERR_ARG, "SetSiCSF: %s", e.c_str());
    const int64_t n = (int64_t)(R.mc.size() + R.bulk.size());
    std::vector<int32_t> xyz((size_t)n * 3), nn((size_t)n * 12);
    int64_t k = 0;
    for (const auto *list : {&R.mc, &R.bulk})
        for (const auto &en : *list) {
            for (int q = 0; q < 3; q++) xyz[(size_t)(3 * k + q)] = en.xyz[q];
            for (int j = 0; j < 4; j++)
                for (int q = 0; q < 3; q++) nn[(size_t)(12 * k + 3 * j + q)] = en.nn[j][q];
            k++;
        }
    return mks_load_lists(h, R.lattcoo.data(), n, xyz.data(), nn.data(), nullptr, nullptr);
}

int mks_batch_init_shape(mks_handle *h, int32_t rep, const char *init_st, const int32_t *lens, const double *params)
{
    if (!h || !init_st || !lens || rep < 0 || rep >= (int)h->reps.size()) return fail(MKS_ERR_ARG, "bad arguments");
    const RepHost &r = h->reps[rep];
    const int lx = r.cfg.lenx, ly = r.cfg.leny, lz = r.cfg.lenz;
    std::string kind(init_st);
    if (kind == "E") return init_sicsf(h, lens);
    mks_shapes::Grid g(lx, ly, lz);
    std::vector<int> temp;
    char msg[160];
    if (int e = mks_shapes::build_shape(g, kind, lens, params, temp, msg, sizeof msg))
        return fail(e == 2 ? MKS_ERR_UNSUPPORTED : MKS_ERR_ARG, "%s", msg);
    int rc = upload_grid(h, rep, g, mks_shapes::ini_rates(kind));
    if (rc) return rc;
    if (kind == "ST")   // the temperatures of SetTrenchSi.f:46-63 as the replica's field
        return set_temperature_impl(h, rep, [&](int, int, int z, int) { return temp[(size_t)z] & 8191; });
    return 0;
}

int mks_batch_init_cad_la(mks_handle *h, int32_t rep, const int8_t *geo, int32_t homogeneous, double len_vac,
                          double len_nuc)
{
    if (!h || !geo || rep < 0 || rep >= (int)h->reps.size()) return fail(MKS_ERR_ARG, "bad arguments");
    const RepHost &r = h->reps[rep];
    if (r.cfg.ncrystal != 1) return fail(MKS_ERR_UNSUPPORTED, "SetCAD is built for NCrystal = 1");
    mks_shapes::Grid g(r.cfg.lenx, r.cfg.leny, r.cfg.lenz);
    mks_shapes::CadLA la;
    la.on = homogeneous >= 0;
    la.homogeneous = homogeneous > 0;
    la.len_vac = len_vac;
    la.len_nuc = len_nuc;
    la.sf = r.cfg.sf;
    mks_shapes::set_cad(g, geo, la);
    return upload_grid(h, rep, g);
}

int mks_batch_init_cad(mks_handle *h, int32_t rep, const int8_t *geo)
{
    return mks_batch_init_cad_la(h, rep, geo, -1, 0.0, 0.0);
}

int mks_batch_init_cad_alloy(mks_handle *h, int32_t rep, const int8_t *geo, double x, uint64_t seed)
{
    if (!h || !geo || rep < 0 || rep >= (int)h->reps.size() || !(x >= 0.0 && x <= 1.0))
        return fail(MKS_ERR_ARG, "bad arguments");
    const RepHost &r = h->reps[rep];
    if (r.cfg.ncrystal < 2 && x > 0.0) return fail(MKS_ERR_ARG, "an alloy needs NCrystal >= 2");
    mks_shapes::Grid g(r.cfg.lenx, r.cfg.leny, r.cfg.lenz);
    mks_shapes::set_cad(g, geo, mks_shapes::CadLA(), x, seed);
    return upload_grid(h, rep, g);
}

int mks_batch_init_points(mks_handle *h, int32_t rep, const int32_t *xyz, const int8_t *species, int64_t n)
{
    if (!h || n < 0 || (n && (!xyz || !species)) || rep < 0 || rep >= (int)h->reps.size())
        return fail(MKS_ERR_ARG, "bad arguments");
    const RepHost &r = h->reps[rep];
    for (int64_t i = 0; i < n; i++) {   // a wall point's species is not read (SetShape.f:58-62)
        const int z = xyz[3 * i + 2];
        if (z > 3 && z < r.cfg.lenz - 4 && species[i] > r.cfg.ncrystal)
            return fail(MKS_ERR_ARG, "point %lld: species %d > NCrystal", (long long)i, species[i]);
    }
    mks_shapes::Grid g(r.cfg.lenx, r.cfg.leny, r.cfg.lenz);
    if (const char *e = mks_shapes::set_points(g, xyz, species, n)) return fail(MKS_ERR_UNSUPPORTED, "SetShape: %s", e);
    return upload_grid(h, rep, g);
}

int mks_init_points(mks_handle *h, const int32_t *xyz, const int8_t *species, int64_t n)
{
    if (!h || h->reps.size() != 1) return fail(MKS_ERR_ARG, "mks_init_points needs a single-replica handle");
    return mks_batch_init_points(h, 0, xyz, species, n);
}

int mks_init_shape(mks_handle *h, const char *init_st, const int32_t *lens, const double *params)
{
    if (!h || h->reps.size() != 1) return fail(MKS_ERR_ARG, "mks_init_shape needs a single-replica handle");
    return mks_batch_init_shape(h, 0, init_st, lens, params);
}

int mks_batch_get_phases(mks_handle *h, int32_t rep, int32_t *coo, int32_t *species)
{
    if (!h || rep < 0 || rep >= (int)h->reps.size() || (!coo && !species)) return fail(MKS_ERR_ARG, "bad arguments");
    const RepHost &r = h->reps[rep];
    const int lx = r.cfg.lenx, ly = r.cfg.leny, lz = r.cfg.lenz;
    const size_t n = (size_t)lz * lx * ly;
    int *d_wall = nullptr;
    int32_t *d_out = nullptr;
    CK(cudaMallocAsync(&d_wall, sizeof(int) * (size_t)r.NZ, h->stream));
    CK(cudaMallocAsync(&d_out, sizeof(int32_t) * n * ((coo && species) ? 2 : 1), h->stream));
    std::vector<int> ones((size_t)r.NZ, 1);
    CK(cudaMemcpyAsync(d_wall, ones.data(), sizeof(int) * ones.size(), cudaMemcpyHostToDevice, h->stream));
    int64_t ns = (int64_t)r.NZ * r.NB * r.NA;
    k_wall_layers<<<(int)std::min<int64_t>(152 * 8, (ns + 255) / 256), 256, 0, h->stream>>>(h->d_reps, rep, h->d_st,
                                                                                               d_wall);
    int32_t *d_coo = coo ? d_out : nullptr, *d_sp = species ? (coo ? d_out + n : d_out) : nullptr;
    k_phases<<<(int)std::min<int64_t>(152 * 16, ((int64_t)n + 255) / 256), 256, 0, h->stream>>>(
        h->d_reps, rep, h->d_st, lx, ly, lz, d_wall, d_coo, d_sp);
    CK(cudaGetLastError());
    if (coo) CK(cudaMemcpyAsync(coo, d_coo, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, h->stream));
    if (species) CK(cudaMemcpyAsync(species, d_sp, sizeof(int32_t) * n, cudaMemcpyDeviceToHost, h->stream));
    cudaFreeAsync(d_wall, h->stream);
    cudaFreeAsync(d_out, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int mks_replay(mks_handle *h, const mks_event *trace, int64_t n)
{
    if (!h || (n > 0 && !trace) || h->reps.size() != 1) return fail(MKS_ERR_ARG, "bad arguments");
    if (n == 0) return 0;
    if (h->stk) {
        int rc = stk_sync(h);
        if (rc) return rc;
        std::string err;
        int64_t done = 0;
        rc = mks_stk::replay(h->stk, trace, n, &done, err);
        return rc ? fail(rc, "replay, event %lld: %s", (long long)done, err.c_str()) : 0;
    }
    mks_event *d_ev = nullptr;
    long long *d_done = nullptr;
    CK(cudaMallocAsync(&d_ev, sizeof(mks_event) * (size_t)n, h->stream));
    CK(cudaMallocAsync(&d_done, sizeof(long long), h->stream));
    CK(cudaMemcpyAsync(d_ev, trace, sizeof(mks_event) * (size_t)n, cudaMemcpyHostToDevice, h->stream));
    k_replay<<<1, 32, 0, h->stream>>>(h->d_reps, h->d_st, d_ev, n, h->d_status, d_done);
    CK(cudaGetLastError());
    long long done = 0;
    CK(cudaMemcpyAsync(&done, d_done, sizeof done, cudaMemcpyDeviceToHost, h->stream));
    cudaFreeAsync(d_ev, h->stream);
    cudaFreeAsync(d_done, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    DevStatus s;
    int rc = read_status(h, s);
    if (rc) return rc;
    if (s.error) {
        CK(cudaMemsetAsync(h->d_status, 0, sizeof(DevStatus), h->stream));
        return fail(s.error, "replay: event %lld is not applicable to the lattice state", done);
    }
    return rescan(h);
}

int mks_replay_noalloc(mks_handle *h, const mks_event *trace, int64_t n)
{
    if (!h || (n > 0 && !trace) || n < 0 || h->reps.size() != 1) return fail(MKS_ERR_ARG, "bad arguments");
    if (n > MKS_REPLAY_NOALLOC_MAX)
        return fail(MKS_ERR_ARG, "mks_replay_noalloc: %lld events exceed the per-call limit of %d; split the trace",
                    (long long)n, MKS_REPLAY_NOALLOC_MAX);
    if (n == 0) return 0;
    if (h->stk) return stk_unsupported("mks_replay_noalloc");
    unsigned char *scratch = h->noalloc_scratch;
    long long *d_done = reinterpret_cast<long long *>(scratch);
    mks_event *d_ev = reinterpret_cast<mks_event *>(scratch + 256);
    // the array keeps the previous call's contents: reset the progress counter
    CK(cudaMemsetAsync(d_done, 0, sizeof(long long), h->stream));
    CK(cudaMemcpyAsync(d_ev, trace, sizeof(mks_event) * (size_t)n, cudaMemcpyHostToDevice, h->stream));
    k_replay<<<1, 32, 0, h->stream>>>(h->d_reps, h->d_st, d_ev, n, h->d_status, d_done);
    CK(cudaGetLastError());
    long long done = 0;
    CK(cudaMemcpyAsync(&done, d_done, sizeof done, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    DevStatus s;
    int rc = read_status(h, s);
    if (rc) return rc;
    if (s.error) {
        CK(cudaMemsetAsync(h->d_status, 0, sizeof(DevStatus), h->stream));
        CK(cudaStreamSynchronize(h->stream));
        return fail(s.error, "replay: event %lld is not applicable to the lattice state", done);
    }
    return rescan(h);
}

int mks_run(mks_handle *h, double tau, int64_t max_windows, int64_t max_events, double max_time,
            int64_t *events_done, double *time_out)
{
    if (!h || h->reps.size() != 1) return fail(MKS_ERR_ARG, "mks_run needs a single-replica handle");
    if (h->stk) {
        int rc = stk_sync(h);
        if (rc) return rc;
        std::string err;
        rc = mks_stk::run(h->stk, tau, max_windows, max_events, max_time, events_done, time_out, err);
        return rc ? fail(rc, "%s", err.c_str()) : 0;
    }
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    unsigned long long e0 = d[0].events;
    rc = run_impl(h, &tau, max_windows, max_events, max_time);
    if (rc) return rc;
    rc = download_reps(h, d);
    if (rc) return rc;
    if (events_done) *events_done = (int64_t)(d[0].events - e0);
    if (time_out) *time_out = d[0].T0;
    return 0;
}

int mks_batch_run(mks_handle *h, const double *tau, int64_t max_windows, int64_t max_events_each,
                  double max_time_each, int64_t *events_total)
{
    if (!h || !tau) return fail(MKS_ERR_ARG, "bad arguments");
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    unsigned long long e0 = 0;
    for (auto &x : d) e0 += x.events;
    rc = run_impl(h, tau, max_windows, max_events_each, max_time_each);
    if (rc) return rc;
    rc = download_reps(h, d);
    if (rc) return rc;
    unsigned long long e1 = 0;
    for (auto &x : d) e1 += x.events;
    if (events_total) *events_total = (int64_t)(e1 - e0);
    return 0;
}

int mks_site_rates(mks_handle *h, int32_t rep, const int32_t *xyz, int64_t n, int32_t *cls, float *rate)
{
    if (!h || n < 0 || (n && (!xyz || !cls || !rate)) || rep < 0 || rep >= (int)h->reps.size())
        return fail(MKS_ERR_ARG, "bad arguments");
    if (h->stk && !h->stk_dirty) return stk_unsupported("mks_site_rates (see mks_get_lists)");
    if (n == 0) return 0;
    int32_t *d_xyz = nullptr, *d_cls = nullptr;
    float *d_rate = nullptr;
    CK(cudaMallocAsync(&d_xyz, sizeof(int32_t) * 3 * (size_t)n, h->stream));
    CK(cudaMallocAsync(&d_cls, sizeof(int32_t) * (size_t)n, h->stream));
    CK(cudaMallocAsync(&d_rate, sizeof(float) * (size_t)n, h->stream));
    CK(cudaMemcpyAsync(d_xyz, xyz, sizeof(int32_t) * 3 * (size_t)n, cudaMemcpyHostToDevice, h->stream));
    int nb = (int)std::min<int64_t>(152 * 8, (n + 255) / 256);
    k_site_rates<<<nb, 256, 0, h->stream>>>(h->d_reps, rep, h->d_st, h->la_on ? h->d_la : nullptr, d_xyz, n, d_cls,
                                            d_rate);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(cls, d_cls, sizeof(int32_t) * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaMemcpyAsync(rate, d_rate, sizeof(float) * (size_t)n, cudaMemcpyDeviceToHost, h->stream));
    cudaFreeAsync(d_xyz, h->stream);
    cudaFreeAsync(d_cls, h->stream);
    cudaFreeAsync(d_rate, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

int mks_class_histogram(mks_handle *h, int64_t *hist, int32_t nclass)
{
    if (!h || !hist || nclass < NCLASS) return fail(MKS_ERR_ARG, "bad arguments");
    if (h->stk && !h->stk_dirty) return stk_unsupported("mks_class_histogram (see mks_get_lists)");
    unsigned long long *d_hist = nullptr;
    CK(cudaMallocAsync(&d_hist, sizeof(unsigned long long) * NCLASS, h->stream));
    CK(cudaMemsetAsync(d_hist, 0, sizeof(unsigned long long) * NCLASS, h->stream));
    class_hist(h, 0, 1, d_hist);
    CK(cudaGetLastError());
    unsigned long long tmp[NCLASS];
    CK(cudaMemcpyAsync(tmp, d_hist, sizeof tmp, cudaMemcpyDeviceToHost, h->stream));
    cudaFreeAsync(d_hist, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    for (int i = 0; i < nclass; i++) hist[i] = i < NCLASS ? (int64_t)tmp[i] : 0;
    return 0;
}

int mks_batch_class_histogram(mks_handle *h, int64_t *hist, int32_t nclass)
{
    if (!h || !hist || nclass < NCLASS) return fail(MKS_ERR_ARG, "bad arguments");
    size_t n = h->reps.size(), nb = sizeof(unsigned long long) * NCLASS;
    unsigned long long *d_hist = nullptr;
    CK(cudaMallocAsync(&d_hist, nb * n, h->stream));
    CK(cudaMemsetAsync(d_hist, 0, nb * n, h->stream));
    class_hist(h, 0, (int)n, d_hist);
    CK(cudaGetLastError());
    std::vector<unsigned long long> tmp(NCLASS * n);
    CK(cudaMemcpyAsync(tmp.data(), d_hist, nb * n, cudaMemcpyDeviceToHost, h->stream));
    cudaFreeAsync(d_hist, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    for (size_t r = 0; r < n; r++)
        for (int i = 0; i < nclass; i++) hist[r * nclass + i] = i < NCLASS ? (int64_t)tmp[r * NCLASS + i] : 0;
    return 0;
}

int mks_get_observables(mks_handle *h, mks_observables *obs)
{
    if (!h || !obs) return fail(MKS_ERR_ARG, "bad arguments");
    if (h->stk) {
        int rc = stk_sync(h);
        if (rc) return rc;
        std::string err;
        rc = mks_stk::observables(h->stk, obs, err);
        return rc ? fail(rc, "%s", err.c_str()) : 0;
    }
    return obs_impl(h, 0, obs);
}

int mks_batch_observables(mks_handle *h, mks_observables *obs)
{
    if (!h || !obs) return fail(MKS_ERR_ARG, "bad arguments");
    for (size_t i = 0; i < h->reps.size(); i++) {
        int rc = obs_impl(h, (int)i, &obs[i]);
        if (rc) return rc;
    }
    return 0;
}

int mks_get_status(mks_handle *h, mks_status *st)
{
    if (!h || !st) return fail(MKS_ERR_ARG, "bad arguments");
    if (h->stk) return mks_stk::status(h->stk, st);
    DevStatus s;
    int rc = read_status(h, s);
    if (rc) return rc;
    std::vector<RepDev> d;
    rc = download_reps(h, d);
    if (rc) return rc;
    memset(st, 0, sizeof *st);
    st->error = s.error;
    st->fallback_tiles = (int64_t)s.fallback;
    st->windows = d[0].window;
    st->active = d[0].active;
    st->stop_reason = d[0].stop_reason;
    return 0;
}

// re-partition every replica with its own width and rescan
int retile(mks_handle *h)
{
    if (h->graph_exec) cudaGraphExecDestroy(h->graph_exec);
    h->graph_exec = nullptr;
    h->graph_windows = 0;
    partition(h);
    int rc = upload_tiles(h);
    if (rc) return rc;
    std::vector<RepDev> d;
    rc = download_reps(h, d);
    if (rc) return rc;
    for (size_t i = 0; i < d.size(); i++) {
        d[i].nqa = h->reps[i].nqa;
        d[i].nqb = h->reps[i].nqb;
        d[i].qshift = h->reps[i].qshift;
        d[i].quad_base = h->reps[i].quad_base;
    }
    rc = upload_reps(h, d);
    if (rc) return rc;
    return rescan(h);
}

int mks_set_tiling(mks_handle *h, int32_t width)
{
    if (!h || width < 4 || width > QMAX) return fail(MKS_ERR_ARG, "tile width must be 4..%d", QMAX);
    for (RepHost &r : h->reps) r.width = width;
    h->tile_width = width;
    return retile(h);
}

int32_t mks_get_tiling(mks_handle *h) { return h ? h->tile_width : 0; }

int mks_batch_set_tiling(mks_handle *h, const int32_t *widths)
{
    if (!h || !widths) return fail(MKS_ERR_ARG, "bad arguments");
    for (size_t i = 0; i < h->reps.size(); i++)
        if (widths[i] < 4 || widths[i] > QMAX) return fail(MKS_ERR_ARG, "replica %zu: tile width must be 4..%d", i, QMAX);
    int wmax = 0;
    for (size_t i = 0; i < h->reps.size(); i++) {
        h->reps[i].width = widths[i];
        wmax = std::max(wmax, (int)widths[i]);
    }
    h->tile_width = wmax;
    return retile(h);
}

int mks_batch_get_tiling(mks_handle *h, int32_t *widths)
{
    if (!h || !widths) return fail(MKS_ERR_ARG, "bad arguments");
    for (size_t i = 0; i < h->reps.size(); i++) widths[i] = h->reps[i].width;
    return 0;
}

int mks_set_colours(mks_handle *h, int32_t ncolour)
{
    if (!h || (ncolour != 0 && ncolour != 3 && ncolour != 4)) return fail(MKS_ERR_ARG, "colours must be 0, 3 or 4");
    if (ncolour == 3)                   // every replica must take the brick tiling
        for (const RepHost &r : h->reps) {
            int t, sh;
            if (!mks_tiling::brick_fits(r.NA, r.width, t, sh))
                return fail(MKS_ERR_ARG, "a %d-site row cannot take the three-colour tiling at width %d", r.NA,
                            r.width);
        }
    h->colours_req = ncolour == 4 ? 4 : 0;
    return retile(h);
}

int32_t mks_get_colours(mks_handle *h) { return h ? h->ncolour : 0; }

// tau = f / r*, with r* the rate of the class that carries the largest share
// of the replica's total rate; f = 0.3 keeps the etch rate of the plain
// Si(001) model inside the 95 % band of the serial reference at 1000-1200 K
// (events per event site per window ~ f).
int mks_suggest_tau(mks_handle *h, double f, double *tau)
{
    if (!h || !tau || !(f > 0.0)) return fail(MKS_ERR_ARG, "bad arguments");
    if (h->stk && !h->stk_dirty) return stk_suggest_tau(h, f, tau);
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    unsigned long long *d_hist = nullptr;
    size_t nb = sizeof(unsigned long long) * NCLASS;
    CK(cudaMallocAsync(&d_hist, nb * h->reps.size(), h->stream));
    CK(cudaMemsetAsync(d_hist, 0, nb * h->reps.size(), h->stream));
    class_hist(h, 0, (int)h->reps.size(), d_hist);
    CK(cudaGetLastError());
    std::vector<unsigned long long> hist(NCLASS * h->reps.size());
    CK(cudaMemcpyAsync(hist.data(), d_hist, nb * h->reps.size(), cudaMemcpyDeviceToHost, h->stream));
    cudaFreeAsync(d_hist, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    for (size_t i = 0; i < h->reps.size(); i++) {
        double best = 0.0, rstar = 0.0;
        for (int c = 1; c < NCLASS; c++) {
            if (c == CLS_ISO || dummy_class(c)) continue;
            double w = (double)hist[i * NCLASS + c] * (double)d[i].rate[c];
            if (w > best) {
                best = w;
                rstar = d[i].rate[c];
            }
        }
        tau[i] = rstar > 0.0 ? f / rstar : 1.0;
    }
    return 0;
}

int mks_frame_sites(mks_handle *h, int32_t kind, uint32_t *idx, int64_t cap, int64_t *n_out)
{
    if (!h || !n_out || (kind != 0 && kind != 1) || h->reps.size() != 1) return fail(MKS_ERR_ARG, "bad arguments");
    if (h->stk && !h->stk_dirty) return stk_unsupported("mks_frame_sites (see mks_get_lists)");
    const RepHost &r = h->reps[0];
    int64_t nunit = (int64_t)r.NZ * r.NB * (r.pitch / 16);
    int nchunk = (int)((nunit + FRAME_UNITS - 1) / FRAME_UNITS);
    unsigned int *d_cnt = nullptr;
    CK(cudaMallocAsync(&d_cnt, sizeof(unsigned int) * nchunk, h->stream));
    if (r.cfg.ncov) kind += 2;
    k_frame_count<<<nchunk, 256, 0, h->stream>>>(h->d_reps, 0, h->d_st, kind, d_cnt);
    CK(cudaGetLastError());
    std::vector<unsigned int> cnt(nchunk);
    CK(cudaMemcpyAsync(cnt.data(), d_cnt, sizeof(unsigned int) * nchunk, cudaMemcpyDeviceToHost, h->stream));
    CK(cudaStreamSynchronize(h->stream));
    std::vector<unsigned long long> off(nchunk);
    unsigned long long tot = 0;
    for (int i = 0; i < nchunk; i++) {
        off[i] = tot;
        tot += cnt[i];
    }
    *n_out = (int64_t)tot;
    if (!idx || (int64_t)tot > cap || tot == 0) {
        cudaFreeAsync(d_cnt, h->stream);
        CK(cudaStreamSynchronize(h->stream));
        return 0;
    }
    unsigned long long *d_off = nullptr;
    uint32_t *d_out = nullptr;
    CK(cudaMallocAsync(&d_off, sizeof(unsigned long long) * nchunk, h->stream));
    CK(cudaMallocAsync(&d_out, sizeof(uint32_t) * tot, h->stream));
    CK(cudaMemcpyAsync(d_off, off.data(), sizeof(unsigned long long) * nchunk, cudaMemcpyHostToDevice, h->stream));
    k_frame_write<<<nchunk, 256, 0, h->stream>>>(h->d_reps, 0, h->d_st, kind, d_off, d_out);
    CK(cudaGetLastError());
    CK(cudaMemcpyAsync(idx, d_out, sizeof(uint32_t) * tot, cudaMemcpyDeviceToHost, h->stream));
    cudaFreeAsync(d_cnt, h->stream);
    cudaFreeAsync(d_off, h->stream);
    cudaFreeAsync(d_out, h->stream);
    CK(cudaStreamSynchronize(h->stream));
    return 0;
}

}  // extern "C"

namespace {

// Fortran Ew.d of the frame headers (WriteMolMolXYZFile.f:166-169)
std::string fortran_e(double v, int w, int d)
{
    char b[64], m[64];
    if (v == 0.0) {
        snprintf(b, sizeof b, "0.%0*dE+00", d, 0);
    } else {
        snprintf(m, sizeof m, "%.*e", d - 1, fabs(v));
        std::string digits;
        const char *p = m;
        digits += *p++;
        if (*p == '.') p++;
        while (*p && *p != 'e') digits += *p++;
        int ex = atoi(p + 1) + 1;
        snprintf(b, sizeof b, "%s0.%sE%c%02d", v < 0 ? "-" : "", digits.c_str(), ex < 0 ? '-' : '+', abs(ex));
    }
    char out[80];
    snprintf(out, sizeof out, "%*s", w, b);
    return out;
}

const char *crystal_symbol(const mks_config &c, int sp)
{   // WriteMolMolXYZFile.f:177-215: species 1 is Si; the second is C, Ge or B
    if (sp == 1) return "Si";
    int z = c.list_crystal[sp - 1];
    return z == 6 ? "C" : (z == 32 ? "Ge" : (z == 5 ? "B" : nullptr));
}

// The frame files of WriteMolMolXYZFile.f:22-406 for an arm-chair stacking
// handle, from its listed sites (every atom and void is listed; walls are
// not written).  Sites follow the reference's z, y, x scan; voids too (the
// reference lists them in ListVoid order).  The SiC wrong-site analysis works
// on a copy, as the compact writer's does.
int stk_write_frame(mks_handle *h, const char *base, double time, int64_t iter, int64_t *num_at_wrong)
{
    const mks_config &c = h->reps[0].cfg;
    std::string err;
    std::vector<mks_stk::Site> all;
    int rc = mks_stk::sites(h->stk, all, err);
    if (rc) return fail(rc, "%s", err.c_str());
    const int64_t lx = c.lenx, ly = c.leny;
    auto key = [&](int64_t x, int64_t y, int64_t z) { return x + lx * (y + ly * z); };
    std::sort(all.begin(), all.end(), [&](const mks_stk::Site &a, const mks_stk::Site &b) {
        return key(a.x, a.y, a.z) < key(b.x, b.y, b.z);
    });
    auto occ = [](uint32_t v) { return (v >> 23) & 1; };
    auto coor = [](uint32_t v) { return (int)((v >> 24) & 7); };
    auto spv = [](uint32_t v) { return (int)((v >> 27) & 7); };
    auto dia = [](int x, int y, int z) {   // SetSi.f:52-57
        if (x % 3 || y % 3 || z % 3) return false;
        int x1 = x / 3, y1 = y / 3, z1 = z / 3;
        if ((x1 & 1) != (y1 & 1) || (x1 & 1) != (z1 & 1)) return false;
        int m = (x1 + y1 + z1) & 3;
        return m == 0 || m == 3;
    };
    const int lz = c.lenz;
    int64_t num_at = 0, noepi = 0, nvoid = 0;
    for (const auto &t : all) {
        uint32_t v = t.word;
        if (t.z >= 1 && t.z <= lz - 1 && occ(v) && coor(v) <= 3) num_at++;
        if (t.z >= 0 && t.z <= lz - 1 && occ(v) && coor(v) == 4 && !dia(t.x, t.y, t.z)) noepi++;
        if (!occ(v) && coor(v) == 4) nvoid++;
    }
    const std::string per = " periodic " + fortran_e(c.sf * c.lenx, 15, 8) + " " + fortran_e(c.sf * c.leny, 15, 8) +
                            " " + fortran_e(c.sf * c.lenz, 15, 8) + "\n";
    auto header = [&](FILE *f, int64_t n) {
        fprintf(f, " %8lld angstroem KMC-time: %s Iter: %12lld\n", (long long)n, fortran_e(time, 15, 8).c_str(),
                (long long)iter);
        fputs(per.c_str(), f);
    };
    auto line = [&](FILE *f, const char *sym, const mks_stk::Site &t) {
        fprintf(f, "%s %10.5f %10.5f %10.5f  \n", sym, c.sf * t.x, c.sf * t.y, c.sf * t.z);
    };
    std::string b(base);
    FILE *f = fopen((b + "_d.xyz").c_str(), "w");          // :96-160, the non-epitaxial bulk
    if (!f) return fail(MKS_ERR_ARG, "cannot write %s_d.xyz", base);
    header(f, noepi);
    for (const auto &t : all) {
        uint32_t v = t.word;
        if (t.z < 0 || t.z > lz - 1 || !occ(v) || coor(v) != 4 || dia(t.x, t.y, t.z)) continue;
        int s = spv(v);
        if (s == 1) line(f, "Ge", t);
        if (s == 2) line(f, "B", t);
        if (s == 3) line(f, "Cl", t);
    }
    fclose(f);
    f = fopen((b + ".xyz").c_str(), "w");
    if (!f) return fail(MKS_ERR_ARG, "cannot write %s.xyz", base);
    header(f, num_at + nvoid);
    for (const auto &t : all) {
        uint32_t v = t.word;
        int s = spv(v);
        if (t.z < 0 || t.z > lz - 1 || s < 1 || s > 3 || coor(v) > 3) continue;
        const char *sym = crystal_symbol(c, s);
        if (!sym || s > c.ncrystal) {
            fclose(f);
            return fail(MKS_ERR_INVARIANT, "ERROR: 2nd crystal specie can only be C/Ge/B");
        }
        line(f, sym, t);
    }
    for (const auto &t : all)
        if (!occ(t.word) && coor(t.word) == 4) line(f, "O", t);
    fclose(f);
    std::unordered_map<int64_t, uint32_t> word;
    word.reserve(all.size() * 2);
    for (const auto &t : all) word[key(t.x, t.y, t.z)] = t.word;
    auto word_at = [&](const int32_t *p) -> uint32_t {
        auto it = word.find(key(p[0], p[1], p[2]));
        return it == word.end() ? 0u : it->second;
    };
    const bool sic = c.ncrystal == 2 && (c.list_crystal[0] == 6 || c.list_crystal[1] == 6 || c.list_crystal[2] == 6);
    f = fopen((b + "_v.xyz").c_str(), "w");                 // :216-260
    if (!f) return fail(MKS_ERR_ARG, "cannot write %s_v.xyz", base);
    fprintf(f, " %8lld angstroem\n", (long long)nvoid);
    fputs(per.c_str(), f);
    for (const auto &t : all) {
        if (occ(t.word) || coor(t.word) != 4) continue;
        if (sic) {
            int sum = 0;
            for (int j = 0; j < 4; j++) sum += spv(word_at(t.nn[j]));
            const char *lbl = sum == 4 ? "Mg %10.5f %10.5f %10.5f # CV (C vacancy)\n"
                            : sum == 8 ? "He %10.5f %10.5f %10.5f # SV (Si vacancy)\n"
                            : sum == 7 ? "Ne %10.5f %10.5f %10.5f # SAV (Si antisite vac)\n"
                            : sum == 5 ? "Be %10.5f %10.5f %10.5f # CAV (C antisite vac)\n"
                            : sum == 6 ? "Ar %10.5f %10.5f %10.5f # XV (near 2C and 2Si)\n" : nullptr;
            if (!lbl) {
                fclose(f);
                return fail(MKS_ERR_INVARIANT, "ERROR: Weird Defect type was formed");
            }
            fprintf(f, lbl, c.sf * t.x, c.sf * t.y, c.sf * t.z);
        } else {
            line(f, "O", t);
        }
    }
    fclose(f);
    if (num_at_wrong) *num_at_wrong = 0;
    if (!sic) return 0;
    // :264-398: bulk atoms (z >= 1) with no neighbour of the other species
    // count as swapped (Si bit 27, C bit 28), then bulk atoms with three are
    // listed
    auto bulk = [&](const mks_stk::Site &t) {
        return t.z >= 1 && t.z <= lz - 1 && occ(t.word) && coor(t.word) == 4 && (t.word & 255) != 113;
    };
    auto other = [&](uint32_t own, uint32_t w) {
        int s = spv(own);
        return s == 1 ? (int)((w >> 28) & 1) : (s == 2 ? (int)((w >> 27) & 1) : 0);
    };
    std::unordered_map<int64_t, uint32_t> sw(word);
    for (const auto &t : all) {
        if (!bulk(t)) continue;
        int nc = 0;
        for (int j = 0; j < 4; j++) nc += other(t.word, word_at(t.nn[j]));
        int s = spv(t.word);
        if (nc == 0 && (s == 1 || s == 2))
            sw[key(t.x, t.y, t.z)] = (t.word & ~(7u << 27)) | ((uint32_t)(s == 1 ? 2 : 1) << 27);
    }
    auto sw_at = [&](const int32_t *p) -> uint32_t {
        auto it = sw.find(key(p[0], p[1], p[2]));
        return it == sw.end() ? 0u : it->second;
    };
    std::vector<std::pair<const mks_stk::Site *, uint32_t>> wrong;
    for (const auto &t : all) {
        if (!bulk(t)) continue;
        uint32_t own = sw[key(t.x, t.y, t.z)];
        int nc = 0;
        for (int j = 0; j < 4; j++) nc += other(own, sw_at(t.nn[j]));
        if (nc == 3) wrong.push_back({&t, own});
    }
    if (num_at_wrong) *num_at_wrong = (int64_t)wrong.size();
    f = fopen((b + "_w.xyz").c_str(), "w");
    if (!f) return fail(MKS_ERR_ARG, "cannot write %s_w.xyz", base);
    fprintf(f, " %8lld angstroem\n", (long long)wrong.size());
    fputs(per.c_str(), f);
    for (const auto &w : wrong) line(f, spv(w.second) == 1 ? "Si" : "C", *w.first);
    fclose(f);
    return 0;
}

}  // namespace

extern "C" {

int mks_write_frame(mks_handle *h, const char *base, double time, int64_t iter, int64_t *num_at_wrong)
{
    if (num_at_wrong) *num_at_wrong = 0;
    if (!h || !base || h->reps.size() != 1) return fail(MKS_ERR_ARG, "mks_write_frame needs a single-replica handle");
    if (h->stk) {
        int rc = stk_sync(h);
        return rc ? rc : stk_write_frame(h, base, time, iter, num_at_wrong);
    }
    const RepHost &r = h->reps[0];
    const mks_config &c = r.cfg;
    const bool cov = c.ncov > 0;
    const int NA = r.NA, NB = r.NB;
    int64_t n0 = 0, n1 = 0;
    int rc = mks_frame_sites(h, 0, nullptr, 0, &n0);
    if (!rc) rc = mks_frame_sites(h, 1, nullptr, 0, &n1);
    if (rc) return rc;
    std::vector<uint32_t> at((size_t)n0), vd((size_t)n1);
    if (n0 && (rc = mks_frame_sites(h, 0, at.data(), n0, &n0))) return rc;
    if (n1 && (rc = mks_frame_sites(h, 1, vd.data(), n1, &n1))) return rc;
    std::vector<uint8_t> st((size_t)mks_state_size(h));
    if ((rc = mks_get_state(h, st.data(), (int64_t)st.size()))) return rc;
    auto site_xyz = [&](int64_t i, double &x, double &y, double &z) {
        int a = (int)(i % NA);
        int64_t q = i / NA;
        int b = (int)(q % NB), z1 = (int)(q / NB);
        x = c.sf * 3.0 * (2 * a + (z1 & 1));
        y = c.sf * 3.0 * (2 * b + (z1 & 1));
        z = c.sf * 3.0 * z1;
    };
    auto nb_byte = [&](int64_t i, int d) -> uint8_t {
        int a = (int)(i % NA);
        int64_t q = i / NA;
        int b = (int)(q % NB), z1 = (int)(q / NB);
        int da, db, dz;
        nb_off(z1 & 1, d, da, db, dz);
        int zz = z1 + dz;
        if (zz < 0 || zz >= r.NZ) return 0;
        return st[((size_t)zz * NB + (size_t)wrapi(b + db, NB)) * NA + (size_t)wrapi(a + da, NA)];
    };
    const std::string per = " periodic " + fortran_e(c.sf * c.lenx, 15, 8) + " " + fortran_e(c.sf * c.leny, 15, 8) +
                            " " + fortran_e(c.sf * c.lenz, 15, 8) + "\n";
    const int64_t layer = (int64_t)NA * NB;
    // the header counts atoms and covered sites from z = 1 (:74-89), the voids all
    int64_t counted = 0;
    for (uint32_t i : at) counted += (int64_t)i >= layer;
    auto header = [&](FILE *f, int64_t n) {
        fprintf(f, " %8lld angstroem KMC-time: %s Iter: %12lld\n", (long long)n, fortran_e(time, 15, 8).c_str(),
                (long long)iter);
        fputs(per.c_str(), f);
    };
    std::string b(base);
    FILE *f = fopen((b + "_d.xyz").c_str(), "w");          // :96-160, cubic stacking: none
    if (!f) return fail(MKS_ERR_ARG, "cannot write %s_d.xyz", base);
    header(f, 0);
    fclose(f);
    f = fopen((b + ".xyz").c_str(), "w");
    if (!f) return fail(MKS_ERR_ARG, "cannot write %s.xyz", base);
    header(f, counted + n1);
    for (uint32_t i : at) {
        double x, y, z;
        site_xyz(i, x, y, z);
        int sp = st[i] & 3;
        const int cz = (cov && sp == COVSP) ? c.list_cov[(st[i] & COV2) ? 1 : 0] : 0;
        const char *sym = (cov && sp == COVSP) ? (cz == 17 ? "Cl" : "H") : crystal_symbol(c, sp);
        if (!sym) {
            fclose(f);
            return fail(MKS_ERR_INVARIANT, "ERROR: 2nd crystal specie can only be C/Ge/B");
        }
        fprintf(f, "%s %10.5f %10.5f %10.5f  \n", sym, x, y, z);
    }
    for (uint32_t i : vd) {
        double x, y, z;
        site_xyz(i, x, y, z);
        fprintf(f, "O %10.5f %10.5f %10.5f  \n", x, y, z);
    }
    fclose(f);
    const bool sic = c.ncrystal == 2 && (c.list_crystal[0] == 6 || c.list_crystal[1] == 6 || c.list_crystal[2] == 6);
    f = fopen((b + "_v.xyz").c_str(), "w");                 // :216-260
    if (!f) return fail(MKS_ERR_ARG, "cannot write %s_v.xyz", base);
    fprintf(f, " %8lld angstroem\n", (long long)n1);
    fputs(per.c_str(), f);
    for (uint32_t i : vd) {
        double x, y, z;
        site_xyz(i, x, y, z);
        if (sic && !cov) {
            int s = 0;
            for (int d = 0; d < 4; d++) s += nb_byte(i, d) & 3;   // species index, 0 on walls
            const char *lbl = s == 4 ? "Mg %10.5f %10.5f %10.5f # CV (C vacancy)\n"
                            : s == 8 ? "He %10.5f %10.5f %10.5f # SV (Si vacancy)\n"
                            : s == 7 ? "Ne %10.5f %10.5f %10.5f # SAV (Si antisite vac)\n"
                            : s == 5 ? "Be %10.5f %10.5f %10.5f # CAV (C antisite vac)\n"
                            : s == 6 ? "Ar %10.5f %10.5f %10.5f # XV (near 2C and 2Si)\n" : nullptr;
            if (!lbl) {
                fclose(f);
                return fail(MKS_ERR_INVARIANT, "ERROR: Weird Defect type was formed");
            }
            fprintf(f, lbl, x, y, z);
        } else {
            fprintf(f, "O %10.5f %10.5f %10.5f  \n", x, y, z);
        }
    }
    fclose(f);
    if (!sic) return 0;
    // :264-398 on a copy: bulk atoms (z >= 1) with no neighbour of the other
    // species are swapped, then bulk atoms with three are listed
    std::vector<uint8_t> sw(st);
    auto is_bulk = [&](uint8_t v) { return v != WALL && (v & 3) != 0 && co_of(v) == 4; };
    auto other = [&](int sp, uint8_t w) { return (sp == 1 && (w & 3) == 2) || (sp == 2 && (w & 3) == 1); };
    for (size_t i = (size_t)layer; i < st.size(); i++) {
        uint8_t v = st[i];
        int sp = v & 3;
        if (!is_bulk(v) || (sp != 1 && sp != 2)) continue;
        int nc = 0;
        for (int d = 0; d < 4; d++) nc += other(sp, nb_byte((int64_t)i, d));
        if (nc == 0) sw[i] = (uint8_t)((v & ~3) | (sp == 1 ? 2 : 1));
    }
    std::vector<size_t> wrong;
    for (size_t i = (size_t)layer; i < sw.size(); i++) {
        uint8_t v = sw[i];
        int sp = v & 3;
        if (!is_bulk(v) || (sp != 1 && sp != 2)) continue;
        int a = (int)(i % NA);
        size_t q = i / NA;
        int bb = (int)(q % NB), z1 = (int)(q / NB);
        int nc = 0;
        for (int d = 0; d < 4; d++) {
            int da, db, dz;
            nb_off(z1 & 1, d, da, db, dz);
            int zz = z1 + dz;
            uint8_t w = (zz < 0 || zz >= r.NZ) ? 0 : sw[((size_t)zz * NB + (size_t)wrapi(bb + db, NB)) * NA + (size_t)wrapi(a + da, NA)];
            nc += other(sp, w);
        }
        if (nc == 3) wrong.push_back(i);
    }
    if (num_at_wrong) *num_at_wrong = (int64_t)wrong.size();
    f = fopen((b + "_w.xyz").c_str(), "w");
    if (!f) return fail(MKS_ERR_ARG, "cannot write %s_w.xyz", base);
    fprintf(f, " %8lld angstroem\n", (long long)wrong.size());
    fputs(per.c_str(), f);
    for (size_t i : wrong) {
        double x, y, z;
        site_xyz((int64_t)i, x, y, z);
        fprintf(f, "%s %10.5f %10.5f %10.5f  \n", (sw[i] & 3) == 1 ? "Si" : "C", x, y, z);
    }
    fclose(f);
    return 0;
}

int mks_get_clock(mks_handle *h, int32_t rep, double *time, int64_t *window, int64_t *events)
{
    if (!h || rep < 0 || rep >= (int)h->reps.size()) return fail(MKS_ERR_ARG, "bad arguments");
    if (h->stk) return mks_stk::clock(h->stk, time, window, events);
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    if (time) *time = d[rep].T0;
    if (window) *window = (int64_t)d[rep].window;
    if (events) *events = (int64_t)d[rep].events;
    return 0;
}

int mks_set_clock(mks_handle *h, int32_t rep, double time, int64_t window, int64_t events)
{
    if (!h || rep < 0 || rep >= (int)h->reps.size() || window < 0 || events < 0 || !(time >= 0.0))
        return fail(MKS_ERR_ARG, "bad arguments");
    if (h->stk) return stk_unsupported("mks_set_clock");
    std::vector<RepDev> d;
    int rc = download_reps(h, d);
    if (rc) return rc;
    d[rep].T0 = time;
    d[rep].window = (unsigned int)window;
    d[rep].events = (unsigned long long)events;
    return upload_reps(h, d);
}

int mks_debug_hold_tile(mks_handle *h, int32_t tile, int64_t spin_limit_cycles)
{
    if (!h || tile < -1 || tile >= (int)h->quads_h.size() || spin_limit_cycles <= 0)
        return fail(MKS_ERR_ARG, "bad arguments");
    h->hold_tile = tile;
    h->spin_limit = spin_limit_cycles;
    return 0;
}

int mks_set_schedule(mks_handle *h, int32_t persistent)
{
    if (!h || (persistent != 0 && persistent != 1)) return fail(MKS_ERR_ARG, "schedule must be 0 or 1");
    h->schedule = persistent;
    return 0;
}

int mks_last_run_stats(mks_handle *h, int64_t *kernel_launches, int64_t *graph_launches, double *kernel_ms,
                       int64_t *phase_launches)
{
    if (!h) return fail(MKS_ERR_ARG, "bad arguments");
    if (kernel_launches) *kernel_launches = h->last_kernels;
    if (graph_launches) *graph_launches = h->last_graphs;
    if (kernel_ms) *kernel_ms = h->last_ms;
    if (phase_launches) *phase_launches = h->last_phase_launches;
    return 0;
}

}  // extern "C"
