// mulskips.e — drop-in replacement of the reference executable, driving the
// GB300 engine through the C ABI (include/mulskips_gpu.h).
//
// Like the reference program (mulskips-source/main.f) it reads ./start.dat,
// builds the initial lattice, runs the KMC loop to the exit condition and
// writes the I%08d.xyz / _d.xyz / _v.xyz / .src frames and movie.mos in the
// current directory, printing the same progress lines (pymulskips greps
// "few MC particles: stop MC", pymulskips/setuprun.py:429-434).
//
// The reference fixes the box at compile time (LenX/LenY/LenZ PARAMETER,
// mulskips-source/modules/defsystem.f:27, rewritten by
// pymulskips/setuprun.py:499-521).  Here the box is read at run time from
// mulskips_box.dat next to this executable ("LenX LenY LenZ"), else from the
// MULSKIPS_BOX environment variable, else 480 480 480.
//
// The loop is the synchronous-sublattice engine: events are counted per
// window, so the Iter exit and the frame schedule are met at the first window
// boundary at or after the requested event count.
#include <ctype.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <algorithm>
#include <string>
#include <vector>
#include <unistd.h>
#include <limits.h>

#include "mulskips_gpu.h"

namespace {

struct Input {
    int ncrystal = 1, ncov = 0;
    int list_crystal[3] = {14, 0, 0};
    int list_cov[3] = {0, 0, 0};
    std::string init_st;
    int len[4] = {120, 120, 120, 120};
    double alloy = 0.0, ptrans_zig = 1.0, sf = 0.4525;
    std::string exit_strategy = "Iter";
    long long max_iter = 2100000000LL, out_molmol = 100000000LL;
    double max_time = 1e8, out_time = 1e7;
    std::string run_type = "R";
    long long idum = 9117116;
    std::string save_final = "F", restart_file, save_coo = "F", coo_file;
    std::vector<double> pE = std::vector<double>(3 * 4096, 0.0);
    std::vector<double> pD = std::vector<double>(9, 0.0);
    std::vector<double> pAbs = std::vector<double>(9, 0.0);   // [coverage species][coor-1]
    std::vector<double> pDes = std::vector<double>(9, 0.0);
    // InitSt ST: angle, Ttop, Tbottom and the probability table rows
    double st_par[3] = {0, 0, 0};
    std::string cad_file;                 // InitSt IN / LA: the LattGeo file
    std::string temp_file;                // InitSt LA: the TempStat file
    double Tm = 0, P0 = 0, sigma = 1, Tflex = 0, len_vac = 0, len_nuc = 0;
    bool homogeneous = true;
    std::vector<int> st_T;
    std::vector<double> st_E, st_D;
};

[[noreturn]] void die(const char *msg)
{
    printf(" %s\n", msg);
    fflush(stdout);
    exit(1);
}

// positional list-directed records of start.dat (main.f:83-212)
struct Records {
    FILE *f;
    std::vector<std::string> toks;
    explicit Records(FILE *fp) : f(fp) {}
    bool line(std::string &out)
    {
        char buf[8192];
        if (!fgets(buf, sizeof buf, f)) return false;
        out = buf;
        while (!out.empty() && (out.back() == '\n' || out.back() == '\r')) out.pop_back();
        return true;
    }
    std::vector<std::string> items(int n)
    {
        std::vector<std::string> r;
        std::string l;
        if (!line(l)) die("start.dat: unexpected end of file");
        toks.clear();
        auto split = [&](const std::string &s) {
            size_t i = 0;
            while (i < s.size()) {
                while (i < s.size() && (isspace((unsigned char)s[i]) || s[i] == ',')) i++;
                size_t j = i;
                while (j < s.size() && !isspace((unsigned char)s[j]) && s[j] != ',') j++;
                if (j > i) toks.push_back(s.substr(i, j - i));
                i = j;
            }
        };
        split(l);
        size_t k = 0;
        while ((int)r.size() < n) {
            if (k >= toks.size()) {
                if (!line(l)) die("start.dat: unexpected end of file");
                toks.clear();
                k = 0;
                split(l);
                continue;
            }
            r.push_back(toks[k++]);
        }
        return r;
    }
};

double real_of(std::string s)
{
    for (auto &c : s)
        if (c == 'd' || c == 'D') c = 'e';
    return strtod(s.c_str(), nullptr);
}

// One block of rate records (SetProbability.f:21-143) into in.pE, pD, pAbs, pDes
void read_rate_block(Records &r, Input &in, bool log)
{
    static const int maxe[4][4] = {{0, 3, 18, 57}, {0, 9, 50, 150}, {0, 19, 100, 288}, {0, 34, 172, 480}};
    std::fill(in.pE.begin(), in.pE.end(), 0.0);
    std::fill(in.pD.begin(), in.pD.end(), 0.0);
    int ne = maxe[in.ncov < 4 ? in.ncov : 0][in.ncrystal];
    if (log) printf(" maxElines %d\n", ne);
    for (int i = 0; i < ne; i++) {
        auto it = r.items(3);
        int s = atoi(it[0].c_str());
        long el = atol(it[1].c_str());
        if (s < 1 || s > in.ncrystal) die("ERROR: 1st index in evap prob must be <= NCrystal");
        int idx[6] = {0, 0, 0, 0, 0, 0};
        int nd = in.ncrystal + in.ncov;
        for (int j = 1; j <= in.ncrystal; j++) {
            long p = 1;
            for (int q = 0; q < nd - j; q++) p *= 10;
            idx[j - 1] = (int)((el / p) % 10);
        }
        for (int j = in.ncrystal + 1; j <= nd; j++) {
            long p = 1;
            for (int q = 0; q < nd - j; q++) p *= 10;
            idx[3 + j - in.ncrystal - 1] = (int)((el / p) % 10);
        }
        int k = (s - 1) * 4096 + idx[0] * 1024 + idx[1] * 256 + idx[2] * 64 + idx[3] * 16 + idx[4] * 4 + idx[5];
        in.pE[k] = real_of(it[2]);
    }
    for (int j = 0; j < in.ncrystal * 3; j++) {
        auto it = r.items(3);
        int s = atoi(it[0].c_str()), el = atoi(it[1].c_str());
        if (s < 1 || s > in.ncrystal || el < 1 || el > 3) die("ERROR: 1st index in depo prob block must be <= NCrystal");
        in.pD[(s - 1) * 3 + el - 1] = real_of(it[2]);
    }
    // absorption, then desorption: NCov*3 records "NCrystal+i  coor  rate"
    // (SetProbability.f:117-140)
    for (int blk = 0; blk < 2; blk++)
        for (int j = 0; j < in.ncov * 3; j++) {
            auto it = r.items(3);
            int s = atoi(it[0].c_str()) - in.ncrystal, el = atoi(it[1].c_str());
            if (s < 1 || s > in.ncov || el < 1 || el > 3) die("ERROR: index in absorption/desorption block");
            (blk ? in.pDes : in.pAbs)[(s - 1) * 3 + el - 1] = real_of(it[2]);
        }
}

Input read_startdat(const char *path)
{
    Input in;
    FILE *f = fopen(path, "r");
    if (!f) die("cannot open start.dat");
    Records r(f);
    auto it = r.items(2);
    in.ncrystal = atoi(it[0].c_str());
    in.ncov = atoi(it[1].c_str());
    if (in.ncrystal < 1 || in.ncrystal > 3) die("ERR NOT IMPLEMENTED: NCrystal must be <= 3");
    it = r.items(in.ncrystal);
    for (int i = 0; i < in.ncrystal; i++) in.list_crystal[i] = atoi(it[i].c_str());
    if (in.ncov > 0) {
        it = r.items(in.ncov);
        for (int i = 0; i < in.ncov; i++) in.list_cov[i] = atoi(it[i].c_str());
    }
    in.init_st = r.items(1)[0].substr(0, 2);
    if (in.init_st == "FF") {
        it = r.items(4);
        for (int i = 0; i < 4; i++) in.len[i] = atoi(it[i].c_str());
    } else if (in.init_st == "ST") {                  // main.f:109-115
        it = r.items(6);
        for (int i = 0; i < 3; i++) in.len[i] = atoi(it[i].c_str());
        for (int i = 0; i < 3; i++) in.st_par[i] = real_of(it[3 + i]);
        printf(" Temperature on top in Kelvin: %.17g\n", in.st_par[1]);
        printf(" Temperature on bottom in Kelvin: %.17g\n", in.st_par[2]);
    } else if (in.init_st == "IN" || in.init_st == "SH") {   // main.f:116-117
        if (!r.line(in.cad_file)) die("start.dat: missing geometry file name");
        while (!in.cad_file.empty() && isspace((unsigned char)in.cad_file.back())) in.cad_file.pop_back();
        while (!in.cad_file.empty() && isspace((unsigned char)in.cad_file.front())) in.cad_file.erase(in.cad_file.begin());
    } else if (in.init_st == "LA") {                  // main.f:118-138
        printf(" ****** MulSKIPs run for laser annealing ******\n");
        if (in.ncov > 0) die("ERR NOT IMPLEMENTED: NCov=0 for LA");
        auto trimmed = [&](std::string &s) {
            if (!r.line(s)) die("start.dat: missing LA file name");
            while (!s.empty() && isspace((unsigned char)s.back())) s.pop_back();
            while (!s.empty() && isspace((unsigned char)s.front())) s.erase(s.begin());
        };
        trimmed(in.cad_file);
        trimmed(in.temp_file);
        in.Tm = real_of(r.items(1)[0]);
        in.P0 = real_of(r.items(1)[0]);
        in.sigma = real_of(r.items(1)[0]);
        in.Tflex = real_of(r.items(1)[0]);
        in.len_vac = real_of(r.items(1)[0]);
        in.len_nuc = real_of(r.items(1)[0]);
        in.homogeneous = r.items(1)[0].substr(0, 1) == "T";
        printf(" Melting temperature in Kelvin: %.17g\n", in.Tm);
    } else {
        it = r.items(3);
        for (int i = 0; i < 3; i++) in.len[i] = atoi(it[i].c_str());
    }
    bool sige = in.ncrystal >= 2 && in.list_crystal[0] == 14 && in.list_crystal[1] == 32 &&
                (in.ncrystal == 2 || in.list_crystal[2] == 5);
    if (sige) in.alloy = real_of(r.items(1)[0]);
    in.ptrans_zig = real_of(r.items(1)[0]);
    in.sf = real_of(r.items(1)[0]);
    in.exit_strategy = r.items(1)[0].substr(0, 4);
    if (in.exit_strategy == "Iter") {
        in.max_iter = atoll(r.items(1)[0].c_str());
        in.out_molmol = atoll(r.items(1)[0].c_str());
    } else if (in.exit_strategy == "Time") {
        in.max_time = real_of(r.items(1)[0]);
        in.out_time = real_of(r.items(1)[0]);
    }
    in.run_type = r.items(1)[0].substr(0, 2);
    in.idum = atoll(r.items(1)[0].c_str());
    in.save_final = r.items(1)[0].substr(0, 2);
    // READ(IPF,'(A)') file names; OPEN drops the blanks around them
    auto trim = [](std::string &t) {
        while (!t.empty() && isspace((unsigned char)t.back())) t.pop_back();
        while (!t.empty() && isspace((unsigned char)t.front())) t.erase(t.begin());
    };
    if (in.save_final == "T") {
        r.line(in.restart_file);
        trim(in.restart_file);
    }
    in.save_coo = r.items(1)[0].substr(0, 2);
    if (in.save_coo == "T") {
        r.line(in.coo_file);
        trim(in.coo_file);
    }
    else if (in.init_st == "LA") die("ERR: SaveCoo flag must be \"T\" for LA simulations!");   // main.f:204-208
    if (in.init_st == "ST") {
        // SetProbabilityFromField.f:23-171: the table file named on the next
        // line: ntemp, nprob, then per temperature its value and one block
        std::string name;
        if (!r.line(name)) die("start.dat: missing probability table file name");
        while (!name.empty() && isspace((unsigned char)name.back())) name.pop_back();
        while (!name.empty() && isspace((unsigned char)name.front())) name.erase(name.begin());
        FILE *tf = fopen(name.c_str(), "r");
        if (!tf) die("cannot open the probability table file");
        Records t(tf);
        int n = atoi(t.items(1)[0].c_str());
        t.items(1);                                   // nprob, unused by the reference too
        if (n < 1 || n > 32) die("ERROR: the GPU engine takes 1..32 table temperatures");
        for (int k = 0; k < n; k++) {
            in.st_T.push_back(atoi(t.items(1)[0].c_str()));
            read_rate_block(t, in, k == 0);
            in.st_E.insert(in.st_E.end(), in.pE.begin(), in.pE.end());
            in.st_D.insert(in.st_D.end(), in.pD.begin(), in.pD.end());
        }
        fclose(tf);
    } else {
        read_rate_block(r, in, true);
    }
    fclose(f);
    return in;
}

void box_size(int &lx, int &ly, int &lz)
{
    lx = ly = lz = 480;
    char exe[PATH_MAX];
    ssize_t n = readlink("/proc/self/exe", exe, sizeof exe - 1);
    if (n > 0) {
        exe[n] = 0;
        std::string d(exe);
        d = d.substr(0, d.rfind('/'));
        FILE *f = fopen((d + "/mulskips_box.dat").c_str(), "r");
        if (f) {
            if (fscanf(f, "%d %d %d", &lx, &ly, &lz) != 3) lx = ly = lz = 480;
            fclose(f);
            return;
        }
    }
    const char *e = getenv("MULSKIPS_BOX");
    if (e) sscanf(e, "%d %d %d", &lx, &ly, &lz);
}

// List-directed READ(unit,*) of a large array (SetCAD.f:58-60,162-170): the
// values are separated by blanks, commas or line breaks and may span several
// records; once the statement has its values the rest of the current record
// is skipped.  Streams the file through a fixed buffer.
struct ListReader {
    FILE *f;
    std::vector<char> buf;
    size_t pos = 0, len = 0;
    explicit ListReader(FILE *fp) : f(fp), buf(1 << 20) {}
    int peek()
    {
        if (pos == len) {
            len = fread(buf.data(), 1, buf.size(), f);
            pos = 0;
            if (len == 0) return EOF;
        }
        return (unsigned char)buf[pos];
    }
    // next value as text; false at the end of the file
    bool token(char *out, size_t cap)
    {
        int c;
        while ((c = peek()) != EOF && (isspace(c) || c == ',')) pos++;
        if (c == EOF) return false;
        size_t n = 0;
        while ((c = peek()) != EOF && !isspace(c) && c != ',') {
            if (n + 1 < cap) out[n++] = (char)c;
            pos++;
        }
        out[n] = 0;
        return n > 0;
    }
    // the rest of the current record
    void end_record()
    {
        int c;
        while ((c = peek()) != EOF && c != '\n') pos++;
        if (c == '\n') pos++;
    }
    // one READ statement of n values, each passed to put(k, text)
    template <class F>
    bool read(size_t n, F put)
    {
        char t[64];
        for (size_t k = 0; k < n; k++) {
            if (!token(t, sizeof t)) return false;
            put(k, t);
        }
        end_record();
        return true;
    }
};

void check(int rc)
{
    if (rc) {
        char buf[512];
        mks_last_error(buf, sizeof buf);
        printf(" ERROR (code %d): %s\n", rc, buf);
        fflush(stdout);
        exit(1);
    }
}

struct Frames {
    mks_handle *h;
    const Input &in;

    bool sic() const
    {
        return in.ncrystal == 2 && (in.list_crystal[0] == 6 || in.list_crystal[1] == 6 || in.list_crystal[2] == 6);
    }
    std::string name(long long iout) const
    {   // GetOutputFileName.f:22-81: first 8 of the 9 digits of 10*Iout
        char d[32];
        snprintf(d, sizeof d, "%09lld", iout * 10);
        return std::string("I") + std::string(d, 8);
    }
    void write(double time, long long iter, long long iout)
    {   // WriteMolMolSource.f:22-112; the xyz files come from mks_write_frame
        // (WriteMolMolXYZFile.f:22-406)
        std::string base = name(iout);
        printf(" %s\n", base.c_str());
        int64_t wrong = 0;
        check(mks_write_frame(h, base.c_str(), time, (int64_t)iter, &wrong));
        if (sic()) printf(" NumAtWrong: %lld\n", (long long)wrong);
        FILE *f;
        f = fopen((base + ".src").c_str(), "w");
        fprintf(f, " load xyz %s.xyz\n color temperature\n set background white\n set boundbox true\n zoom 140\n"
                   " rotate x 41\n rotate y 4\n spacefill 2\n color axes black\n wireframe 2\n color atom green\n"
                   " wireframe 12\n color atom purple\n set bondmode and\n",
                base.c_str());
        fclose(f);
        // movie.mos is first opened at its start (the old content goes), then
        // kept open in APPEND position between frames (WriteMolMolSource.f:74,
        // :104-109); DefAtEnergy.dat gets one blank record per frame, each
        // written from the start of the file (:75, :101-102)
        f = fopen("movie.mos", first ? "w" : "a");
        fprintf(f, " source    %s.src\n write gif %s.gif\n zap\n", base.c_str(), base.c_str());
        fclose(f);
        f = fopen("DefAtEnergy.dat", "w");
        fputs(" \n", f);
        fclose(f);
        first = false;
    }
    bool first = true;
};

}  // namespace

int main()
{
    int lx, ly, lz;
    box_size(lx, ly, lz);
    if (FILE *rt = fopen("Run_time.dat", "w")) fclose(rt);   // FileOpen.f:47, nothing is written to it
    printf(" KMC box size: %d %d %d\n", lx, ly, lz);
    Input in = read_startdat("start.dat");
    printf(" Crystal species (NCrystal= %d ) --> Z: %d %d %d\n", in.ncrystal, in.list_crystal[0], in.list_crystal[1],
           in.list_crystal[2]);
    printf(" KMC Super-Lattice parameter (ang): %.17g\n", in.sf);
    printf(" Exit strategy: %s\n", in.exit_strategy.c_str());
    printf(" IDUM %lld\n", in.idum);
    if (in.ncov > 0) {
        printf(" Coverage species (NCov= %d ) --> Z: %d %d %d\n", in.ncov, in.list_cov[0], in.list_cov[1],
               in.list_cov[2]);
        if (in.ncov > 2 || (in.ncov == 2 && in.ncrystal != 1))
            die("ERR NOT IMPLEMENTED: the GPU engine holds two coverage species with NCrystal = 1, or one");
    }
    const bool shaped = in.init_st == "C" || in.init_st == "S" || in.init_st == "SS" || in.init_st == "I" ||
                        in.init_st == "D" || in.init_st == "Z" || in.init_st == "J" || in.init_st == "K" ||
                        in.init_st == "L" || in.init_st == "T" || in.init_st == "Fw" || in.init_st == "Fa" ||
                        in.init_st == "FF" || in.init_st == "ST" || in.init_st == "E";
    if (in.init_st != "FS" && in.init_st != "F" && in.init_st != "SG" && in.init_st != "IN" && in.init_st != "LA" &&
        in.init_st != "SH" && !shaped)
        die("initialization not_implemented in the GPU engine (A is not: FS, F, Fw, Fa, SG, C, S, SS, I, D, Z, J, K, "
            "L, T, FF, ST, E, IN, SH and LA are)");
    if (in.alloy > 0.0 && in.init_st == "LA")   // SetCAD.f:142,161 read LenSiGe, which nothing sets
        die("ERR: InitSt LA with an alloy fraction > 0 is not built (SetCAD reads an unset LenSiGe there)");
    mks_config cfg;
    memset(&cfg, 0, sizeof cfg);
    cfg.lenx = lx;
    cfg.leny = ly;
    cfg.lenz = lz;
    cfg.ncrystal = in.ncrystal;
    cfg.ncov = in.ncov;
    for (int i = 0; i < 3; i++) cfg.list_crystal[i] = in.list_crystal[i];
    for (int i = 0; i < 3; i++) cfg.list_cov[i] = in.list_cov[i];
    cfg.ptrans_zig = in.ptrans_zig;
    cfg.sf = in.sf;
    cfg.seed = (uint64_t)in.idum;
    // SetSiCSF places atoms off the diamond sites: the explicit-neighbour
    // engine holds them, whatever PtransZig is
    cfg.explicit_nn = in.init_st == "E" ? 1 : 0;
    mks_handle *h = nullptr;
    check(mks_create(&cfg, &h));
    check(mks_set_rates(h, in.pE.data(), in.pD.data()));
    if (in.ncov) check(mks_set_coverage_rates(h, in.pAbs.data(), in.pDes.data()));
    double la_tmax = 0.0;
    if (in.init_st == "LA") {                         // SetT (SetT.f:50-66): TempStat, one READ per layer
        FILE *tf = fopen(in.temp_file.c_str(), "r");
        if (!tf) die("cannot open the temperature file");
        std::vector<int32_t> field((size_t)lx * ly * lz, 10);
        ListReader rd(tf);
        for (int z = 0; z < lz; z++) {
            // list-directed READ of LenX*LenY values (they may span records;
            // the rest of the last record is skipped), x fastest
            bool ok = rd.read((size_t)lx * ly, [&](size_t k, const char *tok) {
                char *e;
                double v = strtod(tok, &e);
                if (e == tok) die("temperature file: not a number");
                const int t = (int)v;                 // INT(LenIn)
                const size_t x = k % (size_t)lx, y = k / (size_t)lx;
                field[(size_t)z + (size_t)lz * (x + (size_t)lx * y)] = t;
                if (t != 10) la_tmax = std::max(la_tmax, (double)t);
            });
            if (!ok) die("temperature file: too few values");
        }
        fclose(tf);
        check(mks_batch_set_field(h, 0, field.data()));
    }
    if ((in.init_st == "IN" || in.init_st == "LA") && in.run_type == "C") {
        // continuation run (SetCAD.f:54-80, main.f:178-182): LattCoo from the
        // checkpoint file named in start.dat, one record of LenX*LenY words
        // per layer z (the dump of main.f:385-403); the lists are rebuilt from
        // it as after a fresh start (SetCAD.f:302-410), the LA temperatures
        // stay those of TempStat
        printf(" ATTENTION!!! You have chosen a continuation run. LattCoo will be read from the following "
               "checkpoint file: %s\n", in.cad_file.c_str());
        FILE *cf = fopen(in.cad_file.c_str(), "r");
        if (!cf) die("cannot open the checkpoint file");
        std::vector<int32_t> lc((size_t)lx * ly * (lz + 1), 0);
        ListReader rd(cf);
        for (int z = 0; z < lz; z++) {
            int32_t *layer = lc.data() + (size_t)lx * ly * z;
            bool ok = rd.read((size_t)lx * ly, [&](size_t k, const char *t) {
                char *e;
                long v = strtol(t, &e, 10);
                if (e == t || *e) die("checkpoint file: not an integer");
                layer[k] = (int32_t)v;
            });
            if (!ok) die("checkpoint file: too few values");
        }
        fclose(cf);
        printf(" Done reading checkpoint file\n");
        check(mks_load_lattice(h, lc.data()));
    } else if (in.init_st == "IN" || in.init_st == "LA") {   // SetCAD.f:155-236: one record per layer z
        printf(" Reading input geometry file: %s\n", in.cad_file.c_str());
        FILE *gf = fopen(in.cad_file.c_str(), "r");
        if (!gf) die("cannot open the geometry file");
        std::vector<int8_t> geo((size_t)lx * ly * lz, 0);
        ListReader rd(gf);
        for (int z = 0; z < lz - 4; z++) {          // the last four layers are walls
            // list-directed READ of LenX*LenY values: the rest of the record is skipped
            int8_t *layer = geo.data() + (size_t)z * lx * ly;
            bool ok = rd.read((size_t)lx * ly, [&](size_t k, const char *t) {
                char *e;
                double v = strtod(t, &e);
                if (e == t) die("geometry file: not a number");
                layer[k] = (int8_t)v;
            });
            if (!ok) die("geometry file: too few values");
        }
        fclose(gf);
        printf(" Done reading input geometry file\n");
        if (in.init_st == "LA")
            check(mks_batch_init_cad_la(h, 0, geo.data(), in.homogeneous ? 1 : 0, in.len_vac, in.len_nuc));
        else if (in.alloy > 0.0 || in.ncrystal > 1)   // SetCAD.f:215-222, the RAND() draw seeded by IDUM here
            check(mks_batch_init_cad_alloy(h, 0, geo.data(), in.alloy, (uint64_t)in.idum));
        else
            check(mks_batch_init_cad(h, 0, geo.data()));
    } else if (in.init_st == "SH") {                  // main.f:281-286, SetShape.f:52-79
        printf(" Reading input geometry file (SHAPE): %s\n", in.cad_file.c_str());
        FILE *sf = fopen(in.cad_file.c_str(), "r");
        if (!sf) die("cannot open the shape file");
        Records pr(sf);
        long long nfilled = atoll(pr.items(1)[0].c_str());
        std::string skip;
        if (nfilled < 0 || !pr.line(skip)) die("shape file: bad header");
        std::vector<int32_t> xyz((size_t)nfilled * 3);
        std::vector<int8_t> sp((size_t)nfilled);
        for (long long i = 0; i < nfilled; i++) {
            auto t = pr.items(4);
            std::string sym = t[0].substr(0, 2);
            sp[i] = sym == "Si" ? 1 : (sym == "C" || sym == "Ge") ? 2 : 0;
            for (int k = 0; k < 3; k++) xyz[3 * i + k] = atoi(t[1 + k].c_str());
        }
        fclose(sf);
        printf(" Done reading input geometry file\n");
        check(mks_init_points(h, xyz.data(), sp.data(), (int64_t)nfilled));
    } else if (in.init_st == "SG") {                  // main.f:240-242: SetSiGex with Len1 rounded to 24
        printf(" Setting up SiGe alloy with fraction = %.17g\n", in.alloy);
        int32_t len1 = in.len[0] - in.len[0] % 24;
        check(mks_batch_init_alloy(h, &len1, &in.alloy, (uint64_t)in.idum));
    } else if (shaped) {                              // main.f:240-278
        int32_t lens[4] = {in.len[0], in.len[1], in.len[2], in.len[3]};
        if (in.init_st == "E")                        // main.f:268-271
            printf(" %d %d %d %d\n", lens[0], lens[1], lens[2], lens[0] - lens[1]);
        check(mks_init_shape(h, in.init_st.c_str(), lens, in.st_par));
    } else {
        int len1 = in.len[0] - in.len[0] % 24;
        check(mks_init_flat(h, in.init_st == "FS" ? 'S' : 'C', len1));
    }
    if (in.init_st == "ST")                           // rates from the table at each site's temperature
        check(mks_batch_set_tabulated(h, (int32_t)in.st_T.size(), in.st_T.data(), in.st_E.data(), in.st_D.data()));
    if (in.init_st == "LA") {                         // the law of Get_Prob.f:127-149 on the static field
        mks_la_params lp;
        memset(&lp, 0, sizeof lp);
        for (int s = 0; s < 3; s++) {
            lp.P0[s] = s == 0 ? (float)in.P0 : 0.f;
            lp.Tm[s] = (float)in.Tm;
            lp.Tflex[s] = (float)in.Tflex;
            lp.sigma[s] = (float)in.sigma;
        }
        lp.w = 1.f;
        lp.L_nm = 1e30f;
        lp.zsurf = 1e30f;
        lp.score = 0;
        lp.liquid_weighting = 0;
        check(mks_batch_set_la(h, &lp, nullptr, nullptr));
    }
    // LA: the window follows the class with the largest share of the rate at
    // the field's hottest temperature (PtransE / PtransD are barriers in eV)
    auto la_tau = [&]() {
        const double kb = 0.00008617330350;           // Get_Prob.f:70
        int64_t hist[MKS_NCLASS] = {0};
        check(mks_class_histogram(h, hist, MKS_NCLASS));
        double rate[MKS_NCLASS] = {0};
        double fe = 0.5 * (1.0 + erf((la_tmax - in.Tflex) / in.sigma));
        const int dep_cls[3] = {1, 3, 4}, occ_cls[3] = {6, 9, 15};   // C1, C2, C3; census 1, 2, 3
        for (int n = 1; n <= 3; n++) {
            double d = in.pD[n - 1], e = in.pE[n * 1024];
            rate[dep_cls[n - 1]] = d != 0.0 ? in.P0 * exp(-d / (kb * in.Tm)) * fe : 0.0;
            rate[occ_cls[n - 1]] = e != 0.0 ? in.P0 * exp(-e / (kb * la_tmax)) : 0.0;
        }
        double best = 0.0, rs = 0.0;
        for (int c = 0; c < MKS_NCLASS; c++)
            if ((double)hist[c] * rate[c] > best) {
                best = (double)hist[c] * rate[c];
                rs = rate[c];
            }
        return rs > 0.0 ? 0.3 / rs : 1e-12;
    };
    mks_observables ob;
    check(mks_get_observables(h, &ob));
    printf(" Atoms,Voids,AdAtoms %lld %lld %lld\n", (long long)(ob.atoms - ob.undercoord), (long long)ob.voids,
           (long long)ob.mc_sites);
    Frames fr{h, in};
    fr.write(0.0, 0, 0);
    bool iter_mode = in.exit_strategy == "Iter";
    long long frame = 0, events = 0;
    double time = 0.0, tau = 0.0;
    int chunk = 16;
    bool few = false;
    for (long long block = 0;; block++) {
        // window factor validated against the serial reference: 0.3 for one
        // crystal species (with or without a coverage species), 0.01 for two
        // or three (fast desorption across tile borders)
        if (block % 4 == 0) {
            if (in.init_st == "LA") tau = la_tau();
            else check(mks_suggest_tau(h, in.ncrystal <= 1 ? 0.3 : 0.01, &tau));
        }
        // Iter mode: the chunk ends at the window that reaches the next
        // output multiple or IterMax, so frames land just past each multiple
        // (one window's events at most) instead of a whole chunk later
        int64_t cap = 0;
        if (iter_mode) {
            long long next = in.max_iter;
            if (in.out_molmol > 0) next = std::min(next, (frame + 1) * in.out_molmol);
            cap = next > events ? next - events : 1;
        }
        int64_t ev = 0;
        check(mks_run(h, tau, chunk, cap, 0.0, &ev, &time));
        events += ev;
        mks_status st;
        check(mks_get_status(h, &st));
        if (st.stop_reason == 1) {
            check(mks_get_observables(h, &ob));
            printf(" few MC particles: stop MC %lld %lld\n", events, (long long)ob.mc_sites);
            few = true;
            break;
        }
        if (iter_mode) {
            while (in.out_molmol > 0 && events >= (frame + 1) * in.out_molmol && events < in.max_iter) {
                frame++;
                fr.write(time, events, frame);
                check(mks_get_observables(h, &ob));
                printf(" Iter, Time %lld %.17g\n", events, time);
                printf(" NatNvoidNad %lld %lld %lld\n", (long long)(ob.atoms - ob.undercoord), (long long)ob.voids,
                       (long long)ob.mc_sites);
            }
            if (events >= in.max_iter) break;
        } else {
            // main.f:324-330: a frame whenever Time passes the next output
            // time, checked before the exit test of :365
            while (in.out_time > 0 && time >= (frame + 1) * in.out_time) {
                frame++;
                fr.write(time, events, frame);
                printf(" Iter, Time %lld %.17g\n", events, time);
            }
            if (time > in.max_time) break;
        }
    }
    // main.f:374-377 numbers the final frame Iter/OutMolMol; the reference
    // stops at IterMax exactly, the window that crosses it may overshoot
    if (iter_mode)
        fr.write(time, events, in.out_molmol > 0 ? std::min(events, in.max_iter) / in.out_molmol : 0);
    else
        fr.write(time, events, frame);
    check(mks_get_observables(h, &ob));
    printf(" Iter, Time %lld %.17g\n", events, time);
    printf(" NatNvoidNad %lld %lld %lld\n", (long long)(ob.atoms - ob.undercoord), (long long)ob.voids,
           (long long)ob.mc_sites);
    if (in.save_final == "T" || in.save_coo == "T") {
        std::vector<int32_t> lc((size_t)lx * ly * (lz + 1));
        check(mks_get_lattice(h, lc.data()));
        if (in.save_final == "T") {   // main.f:385-403, one plane per record
            FILE *f = fopen(in.restart_file.c_str(), "w");
            for (int z = 0; z < lz; z++) {
                for (size_t k = 0; k < (size_t)lx * ly; k++) fprintf(f, " %d", lc[(size_t)lx * ly * z + k]);
                fputc('\n', f);
            }
            fclose(f);
        }
        if (in.save_coo == "T") {     // main.f:407-430, FORMAT(500000I4)
            FILE *f = fopen(in.coo_file.c_str(), "w");
            for (int z = 0; z < lz; z++) {
                for (size_t k = 0; k < (size_t)lx * ly; k++) {
                    int32_t v = lc[(size_t)lx * ly * z + k];
                    int out = 0;
                    if ((v & 255) == 113) out = 10;
                    else if ((v >> 23) & 1) out = (v >> 24) & 7;
                    fprintf(f, "%4d", out);
                }
                fputc('\n', f);
            }
            fclose(f);
        }
    }
    mks_destroy(h);
    (void)few;
    return 0;
}
