// Test helper: applies the oracle's event trace to the one-byte lattice
// rules of mulskips_gb300/csrc/lattice.cuh compiled for the host, and
// compares every site byte and every MC site's rate class with the oracle
// after each chunk.  Prints one line per chunk; exit code 0 on full parity.
// usage: compact_check START.DAT NUMBERS LEN BOXSIDE KIND(S|C) EVENTS CHUNK
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <vector>
#include "../../oracle/mks_oracle.h"
#include "../../mulskips_gb300/csrc/lattice.cuh"
using namespace mks;

struct Lat {
    int NA, NB, NZ;
    std::vector<uint8_t> v;
    uint8_t get(int a, int b, int z) const
    {
        if (z < 0 || z >= NZ) return 0;
        a = (a % NA + NA) % NA;
        b = (b % NB + NB) % NB;
        return v[((size_t)z * NB + b) * NA + a];
    }
    void put(int a, int b, int z, uint8_t x)
    {
        if (z < 0 || z >= NZ) return;
        a = (a % NA + NA) % NA;
        b = (b % NB + NB) % NB;
        v[((size_t)z * NB + b) * NA + a] = x;
    }
};

int main(int argc, char **argv)
{
    if (argc < 8) return 2;
    int len1 = atoi(argv[3]), side = atoi(argv[4]);
    bool sic = argv[5][0] == 'C';
    long long total = atoll(argv[6]), chunk = atoll(argv[7]);
    ora_t *o = ora_create(argv[1], argv[2], side, side, side, 0);
    if (!o || ora_init(o)) {
        printf("oracle: %s\n", ora_last_error());
        return 1;
    }
    // census enumeration of lattice.cuh vs the oracle's class export
    int k = 0;
    for (int t = 1; t <= 3; t++)
        for (int a = t; a >= 0; a--)
            for (int b = t - a; b >= 0; b--, k++)
                if (census_index(a, b, t - a - b) != k) {
                    printf("census enumeration mismatch\n");
                    return 1;
                }
    Lat L{side / 6, side / 6, side / 3 + 1, {}};
    L.v.assign((size_t)L.NA * L.NB * L.NZ, 0);
    for (int z = 0; z < L.NZ; z++)
        for (int b = 0; b < L.NB; b++)
            for (int a = 0; a < L.NA; a++)
                if (((a + b + (z >> 1)) & 1) == 0) L.v[((size_t)z * L.NB + b) * L.NA + a] = flat_init_state(z, side, len1 - len1 % 24, sic);
    std::vector<uint8_t> ref(L.v.size());
    std::vector<int32_t> cls(1 << 22);
    std::vector<double> rate(1 << 22);
    double pE[3 * 4096], pD[9];
    ora_get_rates(o, pE, pD);
    ora_trace_enable(o, 1);
    long long done = 0;
    int bad_total = 0;
    for (;;) {
        long long off = ora_compact_state(o, ref.data());
        long long mism = 0;
        for (size_t i = 0; i < ref.size(); i++) mism += ref[i] != L.v[i];
        // class histogram of the model vs the oracle's own
        std::vector<long long> hm(NCLASS, 0), ho(NCLASS, 0);
        for (int z = 0; z < L.NZ; z++)
            for (int b = 0; b < L.NB; b++)
                for (int a = 0; a < L.NA; a++)
                    if (((a + b + (z >> 1)) & 1) == 0) hm[site_class(L, a, b, z)]++;
        long long nmc = ora_mc_classes(o, cls.data(), rate.data(), (long long)cls.size());
        long long ratebad = 0;
        for (long long i = 0; i < nmc; i++) {
            ho[cls[i]]++;
            int c = cls[i];
            double r = -1;
            if (c >= 1 && c <= 4 && c != 2) {
                int co = c == 1 ? 1 : c - 1;
                r = pD[co - 1] + pD[3 + co - 1] + pD[6 + co - 1];
            } else if (c == 2) {
                r = (double)1.e-8f;
            } else if (c == CLS_C1I) {
                r = (double)1.e-6f;
            } else if (c >= CLS_OCC0) {
                int q = c - CLS_OCC0, sp = q / NCENSUS + 1, ci = q % NCENSUS, kk = 0;
                for (int t = 1; t <= 3; t++)
                    for (int a = t; a >= 0; a--)
                        for (int b = t - a; b >= 0; b--, kk++)
                            if (kk == ci) r = pE[(sp - 1) * 4096 + a * 1024 + b * 256 + (t - a - b) * 64];
            }
            if (c != CLS_ISO && r != rate[i]) ratebad++;
        }
        long long hbad = 0;
        for (int c = 1; c < NCLASS; c++) hbad += hm[c] != ho[c];
        printf("events %lld state_mismatch %lld hist_mismatch %lld rate_mismatch %lld offgrid %lld mc %lld\n", done,
               mism, hbad, ratebad, off, nmc);
        bad_total += (mism != 0) + (hbad != 0) + (ratebad != 0) + (off != 0);
        if (done >= total) break;
        ora_trace_clear(o);
        int r = ora_run(o, chunk, NULL);
        if (r < 0) {
            printf("oracle: %s\n", ora_last_error());
            return 1;
        }
        const ora_event_t *t = ora_trace(o);
        long long n = ora_trace_len(o);
        for (long long i = 0; i < n; i++) {
            int z1 = t[i].z / 3, a = (t[i].x / 3) >> 1, b = (t[i].y / 3) >> 1;
            Touched tc;
            int e = t[i].itrans <= 3 ? apply_deposition(L, a, b, z1, t[i].itrans, tc) : apply_evaporation(L, a, b, z1, tc);
            if (e) {
                printf("rule error %d at event %lld\n", e, done + i);
                return 1;
            }
        }
        done += n;
        if (r) {
            printf("oracle stopped (code %d) after %lld events\n", r, done);
            total = done;
        }
    }
    ora_destroy(o);
    return bad_total ? 1 : 0;
}
