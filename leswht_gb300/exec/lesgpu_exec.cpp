// lesgpu_exec: the drop-in for the reference's solver_exec.
//
// Run from a 02_solver-style directory, it follows solver.f90:26-195 --
// readsettings, readbcs (boundary.input + ../output/ibmpre/ibmpre_prdic.bin),
// readgeom (the grid.bin named in settings.input), the pre-processing tables
// (ibmpre_fcpts, _fcpts_t, _nutzero, _wallfdvm, _conjg, _omega), prefld
// (IREAD = 1) or makefld (IREAD = 0) -- then the time loop, with the whole
// step on the GPU through the C ABI of include/lesgpu.h, and writes the
// reference's outputs: ../output/ftr/{fhist,fcmfr,ftemp,fcdcl,fheatflux,
// ftime}.dat, ../output/field/fld%07d (writefield) and
// ../output/field_avg/fav%07d-%07d (field_avg).
//
// The reference links its body function and its Poisson solver at compile
// time; this driver reads them, and the arithmetic form, from body.input
// ("KIND CX CY CZ R P0 POISSON PRECISION" header, one value line).
#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include <sys/stat.h>

#include "../../include/lesgpu.h"

namespace {

[[noreturn]] void die(const std::string &msg) {
    fprintf(stderr, "lesgpu_exec: %s\n", msg.c_str());
    exit(1);
}

void check(int rc, const char *what) {
    if (rc != 0) die(std::string(what) + ": " + lesgpu_strerror(rc));
}

// ---------------------------------------------------------------- list-directed reads
// One Fortran `read (u, *) a, b, ...`: starts on a new record (line), takes
// as many lines as it needs, drops the rest of the last one.
struct ListReader {
    std::ifstream in;
    std::string path;
    explicit ListReader(const std::string &p) : in(p), path(p) {
        if (!in) die("cannot open " + p);
    }
    std::vector<std::string> items(size_t n) {
        std::vector<std::string> out;
        std::string line;
        while (out.size() < n) {
            if (!std::getline(in, line)) die(path + ": unexpected end of file");
            size_t i = 0;
            while (i < line.size() && out.size() < n) {
                while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == ',' || line[i] == '\r')) i++;
                if (i >= line.size()) break;
                if (line[i] == '"' || line[i] == '\'') {
                    char q = line[i++];
                    size_t j = line.find(q, i);
                    if (j == std::string::npos) j = line.size();
                    out.push_back(line.substr(i, j - i));
                    i = j + 1;
                } else {
                    size_t j = i;
                    while (j < line.size() && line[j] != ' ' && line[j] != '\t' && line[j] != ',' && line[j] != '\r') j++;
                    out.push_back(line.substr(i, j - i));
                    i = j;
                }
            }
        }
        return out;
    }
    void skip() { items(1); }
};

double to_d(std::string s) {
    for (char &ch : s)
        if (ch == 'd' || ch == 'D') ch = 'E';
    return strtod(s.c_str(), nullptr);
}
int64_t to_i(const std::string &s) { return strtoll(s.c_str(), nullptr, 10); }

// whitespace-separated numbers of a whole text file
std::vector<double> read_all_numbers(const std::string &p) {
    std::ifstream in(p);
    if (!in) die("cannot open " + p);
    std::vector<double> v;
    std::string tok;
    while (in >> tok) v.push_back(to_d(tok));
    return v;
}

bool exists(const std::string &p) {
    std::ifstream in(p);
    return (bool)in;
}

// ---------------------------------------------------------------- Fortran records
void write_records(const std::string &path, const std::vector<std::vector<char>> &recs) {
    FILE *f = fopen(path.c_str(), "wb");
    if (!f) die("cannot write " + path);
    for (const auto &r : recs) {
        int32_t n = (int32_t)r.size();
        fwrite(&n, 4, 1, f);
        fwrite(r.data(), 1, r.size(), f);
        fwrite(&n, 4, 1, f);
    }
    fclose(f);
}
std::vector<std::vector<char>> read_records(const std::string &path) {
    FILE *f = fopen(path.c_str(), "rb");
    if (!f) die("cannot open " + path);
    std::vector<std::vector<char>> out;
    int32_t n;
    while (fread(&n, 4, 1, f) == 1) {
        std::vector<char> r((size_t)n);
        if (fread(r.data(), 1, r.size(), f) != r.size()) die(path + ": truncated record");
        int32_t n2;
        if (fread(&n2, 4, 1, f) != 1 || n2 != n) die(path + ": bad record marker");
        out.push_back(std::move(r));
    }
    fclose(f);
    return out;
}
template <class T> void put(std::vector<char> &r, T v) {
    const char *p = (const char *)&v;
    r.insert(r.end(), p, p + sizeof(T));
}
template <class T> T get(const std::vector<char> &r, size_t &pos) {
    T v;
    memcpy(&v, r.data() + pos, sizeof(T));
    pos += sizeof(T);
    return v;
}

// ---------------------------------------------------------------- the case
struct Grid {
    int64_t n1, n2, n3, n1m, n2m, n3m;
    double xl, yl, zl;
    std::vector<double> x, y, z, xmp, ymp, zmp, c2c[3], c2ci[3], f2f[3], f2fi[3];
    std::vector<int64_t> pv[3], mv[3], fl[3], fu[3];
    size_t nt() const { return (size_t)(n1 + 1) * (n2 + 1) * (n3 + 1); }
    size_t ix(int64_t i, int64_t j, int64_t k) const { return (size_t)i + (n1 + 1) * ((size_t)j + (n2 + 1) * (size_t)k); }
};

// readgeom, misc_init.f90:204-251
Grid readgeom(const std::string &path) {
    std::vector<double> v = read_all_numbers(path);
    size_t p = 0;
    auto take = [&](size_t n) {
        if (p + n > v.size()) die(path + ": truncated");
        std::vector<double> out(v.begin() + p, v.begin() + p + n);
        p += n;
        return out;
    };
    Grid g;
    auto h = take(3);
    g.n1 = (int64_t)h[0]; g.n2 = (int64_t)h[1]; g.n3 = (int64_t)h[2];
    h = take(3);
    g.n1m = (int64_t)h[0]; g.n2m = (int64_t)h[1]; g.n3m = (int64_t)h[2];
    h = take(3);
    g.xl = h[0]; g.yl = h[1]; g.zl = h[2];
    g.x = take(g.n1); g.y = take(g.n2); g.z = take(g.n3);
    const int64_t nm[3] = {g.n1m, g.n2m, g.n3m}, n[3] = {g.n1, g.n2, g.n3};
    auto ivec = [&](int64_t cnt) {
        auto d = take(cnt);
        std::vector<int64_t> o(d.size());
        for (size_t q = 0; q < d.size(); q++) o[q] = (int64_t)llround(d[q]);
        return o;
    };
    for (int a = 0; a < 3; a++) g.pv[a] = ivec(nm[a]);
    for (int a = 0; a < 3; a++) g.mv[a] = ivec(nm[a]);
    for (int a = 0; a < 3; a++) g.fl[a] = ivec(nm[a]);
    for (int a = 0; a < 3; a++) g.fu[a] = ivec(nm[a]);
    for (int a = 0; a < 3; a++) g.c2c[a] = take(n[a] + 1);
    for (int a = 0; a < 3; a++) g.c2ci[a] = take(n[a] + 1);
    for (int a = 0; a < 3; a++) g.f2f[a] = take(n[a] + 1);
    for (int a = 0; a < 3; a++) g.f2fi[a] = take(n[a] + 1);
    g.xmp = take(g.n1 + 1); g.ymp = take(g.n2 + 1); g.zmp = take(g.n3 + 1);
    return g;
}

double funcbody(const lesgpu_body &b, double x, double y, double z) {
    switch (b.kind) {
    case LESGPU_BODY_CHANNEL: return (1.0 + b.p0) - fabs(y);
    case LESGPU_BODY_CYLINDER: return sqrt((x - b.cx) * (x - b.cx) + (y - b.cy) * (y - b.cy)) - b.r;
    case LESGPU_BODY_SPHERE:
        return sqrt((x - b.cx) * (x - b.cx) + (y - b.cy) * (y - b.cy) + (z - b.cz) * (z - b.cz)) - b.r;
    case LESGPU_BODY_SQUARE: return fmax(fabs(x - b.cx), fabs(y - b.cy)) - b.r;
    default: return 1.0;
    }
}

struct Tables {
    int64_t nintp[4] = {0, 0, 0, 0}, nbody[4] = {0, 0, 0, 0};
    std::vector<int64_t> fc[4], ix[4], inz, jnz, knz, nwall, omega;
    std::vector<double> gf[4], cstar, kstar;
    int64_t nzero = 0;
};

// alloinit / ibmpreread / nutzeroread / conjgread, misc_init.f90:253-440
Tables read_tables(const lesgpu_config &c, const Grid &g) {
    Tables t;
    const std::string d = "../output/ibmpre/";
    auto read_list = [&](const std::string &file, int l0, int nl) {
        std::vector<double> v = read_all_numbers(d + file);
        size_t p = 0;
        for (int l = l0; l < l0 + nl; l++) t.nintp[l] = (int64_t)v[p++];
        for (int l = l0; l < l0 + nl; l++) t.nbody[l] = t.nintp[l] + (int64_t)v[p++];
        for (int l = l0; l < l0 + nl; l++) {
            t.fc[l].resize(3 * t.nbody[l]);
            for (auto &e : t.fc[l]) e = (int64_t)llround(v[p++]);
        }
        for (int l = l0; l < l0 + nl; l++) {
            t.ix[l].resize(3 * t.nintp[l]);
            for (auto &e : t.ix[l]) e = (int64_t)llround(v[p++]);
        }
        for (int l = l0; l < l0 + nl; l++) {
            t.gf[l].resize(27 * t.nintp[l]);
            for (auto &e : t.gf[l]) e = v[p++];
        }
        if (p > v.size()) die(file + ": truncated");
    };
    read_list("ibmpre_fcpts.bin", 0, 3);
    if (c.ihtrans == 1 && exists(d + "ibmpre_fcpts_t.bin")) read_list("ibmpre_fcpts_t.bin", 3, 1);
    const size_t ncell = (size_t)g.n1m * g.n2m * g.n3m;
    if (c.iles == 1) {
        std::vector<double> v = read_all_numbers(d + "ibmpre_nutzero.bin");
        t.nzero = (int64_t)v.at(0);
        for (int64_t q = 0; q < t.nzero; q++) t.inz.push_back((int64_t)v.at(1 + q));
        for (int64_t q = 0; q < t.nzero; q++) t.jnz.push_back((int64_t)v.at(1 + t.nzero + q));
        for (int64_t q = 0; q < t.nzero; q++) t.knz.push_back((int64_t)v.at(1 + 2 * t.nzero + q));
        std::vector<double> w = read_all_numbers(d + "ibmpre_wallfdvm.bin");
        if (w.size() < ncell) die("ibmpre_wallfdvm.bin: truncated");
        t.nwall.resize(ncell);
        for (size_t q = 0; q < ncell; q++) t.nwall[q] = (int64_t)w[q];
    }
    if (c.iconjg == 1) {
        std::vector<double> v = read_all_numbers(d + "ibmpre_conjg.bin");
        if (v.size() < 7 * ncell) die("ibmpre_conjg.bin: truncated");
        t.cstar.assign(v.begin(), v.begin() + ncell);
        t.kstar.assign(v.begin() + ncell, v.begin() + 7 * ncell);
        if (exists(d + "ibmpre_omega.bin")) {
            std::vector<double> o = read_all_numbers(d + "ibmpre_omega.bin");
            t.omega.resize(ncell);
            for (size_t q = 0; q < ncell; q++) t.omega[q] = (int64_t)o.at(q);
        }
    }
    return t;
}

struct State {
    std::vector<double> u, v, w, p, t;
    int64_t ihist = 0, m = 0;
    double time = 0, dt = 0;
};

// prefld, misc_init.f90:610-786 (the ghost copies are redone on the device
// by the first step's boundary updates as in the reference's prdic calls)
State prefld(const std::string &path, lesgpu_config &c, const Grid &g) {
    auto r = read_records(path);
    if (r.size() < 9) die(path + ": too few records");
    size_t pos = 0;
    int64_t n1 = get<int64_t>(r[0], pos), n2 = get<int64_t>(r[0], pos), n3 = get<int64_t>(r[0], pos);
    if (n1 != g.n1 || n2 != g.n2 || n3 != g.n3) die("PREVIOUS FIELD DOES NOT MATCH WITH THE GRID SYSTEM.");
    State s;
    pos = 0;
    s.ihist = get<int64_t>(r[1], pos); s.m = get<int64_t>(r[1], pos);
    s.time = get<double>(r[1], pos); s.dt = get<double>(r[1], pos);
    // the periodicity, boundary kinds and ICH / ICONJG stored with the field
    // replace those of boundary.input and ibmpre_prdic.bin
    if (r[2].size() < 24 || r[3].size() < 48 || r[4].size() < 16) die(path + ": short header records");
    pos = 0;
    c.xprdic = get<int64_t>(r[2], pos); c.yprdic = get<int64_t>(r[2], pos); c.zprdic = get<int64_t>(r[2], pos);
    pos = 16;   // bc_xbtm, bc_xtop follow from xprdic
    c.bc_ybtm = get<int64_t>(r[3], pos); c.bc_ytop = get<int64_t>(r[3], pos);
    c.bc_zbtm = get<int64_t>(r[3], pos); c.bc_ztop = get<int64_t>(r[3], pos);
    pos = 0;
    c.ich = get<int64_t>(r[4], pos); c.iconjg = get<int64_t>(r[4], pos);
    const size_t nt = g.nt();
    s.u.assign(nt, 0.0); s.v.assign(nt, 0.0); s.w.assign(nt, 0.0); s.p.assign(nt, 0.0);
    s.t.assign(nt, c.tsol_i);
    auto fill = [&](const std::vector<char> &rec, std::vector<double> &a, int64_t i0, int64_t i1, int64_t j0,
                    int64_t j1, int64_t k0, int64_t k1) {
        size_t need = (size_t)(i1 - i0 + 1) * (j1 - j0 + 1) * (k1 - k0 + 1) * 8;
        if (rec.size() != need) die(path + ": record size does not match the grid");
        size_t q = 0;
        for (int64_t k = k0; k <= k1; k++)
            for (int64_t j = j0; j <= j1; j++)
                for (int64_t i = i0; i <= i1; i++) {
                    double x;
                    memcpy(&x, rec.data() + 8 * q++, 8);
                    a[g.ix(i, j, k)] = x;
                }
    };
    fill(r[5], s.u, 1, g.n1, 0, g.n2, 0, g.n3);
    fill(r[6], s.v, 0, g.n1, 1, g.n2, 0, g.n3);
    fill(r[7], s.w, 0, g.n1, 0, g.n2, 1, g.n3);
    fill(r[8], s.p, 1, g.n1m, 1, g.n2m, 1, g.n3m);
    if (c.ihtrans == 1) {
        if (r.size() < 10) die(path + ": no temperature record");
        fill(r[9], s.t, 1, g.n1m, 1, g.n2m, 1, g.n3m);
    }
    if (c.ipzero == 1) std::fill(s.p.begin(), s.p.end(), 0.0);
    // periodic ghost copies of prefld (misc_init.f90:655-786)
    auto per = [&](std::vector<double> &a, int dir, int64_t lo0, int64_t hi0, int64_t lo1, int64_t hi1) {
        for (int64_t b = lo1; b <= hi1; b++)
            for (int64_t q = lo0; q <= hi0; q++) {
                if (dir == 0) { a[g.ix(0, q, b)] = a[g.ix(g.n1m, q, b)]; a[g.ix(g.n1, q, b)] = a[g.ix(1, q, b)]; }
                if (dir == 1) { a[g.ix(q, 0, b)] = a[g.ix(q, g.n2m, b)]; a[g.ix(q, g.n2, b)] = a[g.ix(q, 1, b)]; }
                if (dir == 2) { a[g.ix(q, b, 0)] = a[g.ix(q, b, g.n3m)]; a[g.ix(q, b, g.n3)] = a[g.ix(q, b, 1)]; }
            }
    };
    if (c.xprdic == 1) {
        per(s.u, 0, 0, g.n2, 0, g.n3); per(s.v, 0, 1, g.n2, 0, g.n3); per(s.w, 0, 0, g.n2, 1, g.n3);
        if (c.ihtrans == 1) per(s.t, 0, 0, g.n2, 0, g.n3);
    }
    if (c.yprdic == 1) {
        per(s.u, 1, 1, g.n1, 0, g.n3); per(s.v, 1, 0, g.n1, 0, g.n3); per(s.w, 1, 0, g.n1, 1, g.n3);
        if (c.ihtrans == 1) per(s.t, 1, 0, g.n1, 0, g.n3);
    }
    if (c.zprdic == 1) {
        per(s.u, 2, 1, g.n1, 0, g.n2); per(s.v, 2, 0, g.n1, 1, g.n2); per(s.w, 2, 0, g.n1, 0, g.n2);
        if (c.ihtrans == 1) per(s.t, 2, 0, g.n1, 0, g.n2);
    }
    return s;
}

// makefld, misc_init.f90:443-606: the inflow profile in the fluid, u = 0 on
// the no-slip walls, T = TSOL_I in the solid and TFLU_I (or u/Pr with
// IDECOMP = 1) in the fluid, then the thermal boundary values.  The i = 0
// column evaluates funcbody at x(0), which lies outside x(1:n1) in the
// reference; here it is the mirrored gridline 2 x(1) - x(2).  The random
// EPS_PTR perturbation (addperturb) is not applied.
State makefld(const lesgpu_config &c, const Grid &g) {
    State s;
    const size_t nt = g.nt();
    s.u.assign(nt, 0.0); s.v.assign(nt, 0.0); s.w.assign(nt, 0.0); s.p.assign(nt, 0.0);
    s.t.assign(nt, c.tsol_i);
    auto xg = [&](int64_t i) { return i >= 1 ? g.x[i - 1] : 2.0 * g.x[0] - g.x[1]; };
    for (int64_t k = 0; k <= g.n3; k++)
        for (int64_t j = 0; j <= g.n2; j++)
            for (int64_t i = 0; i <= g.n1; i++) {
                const double y = g.ymp[j];
                double val = 0.0;
                if (funcbody(c.body, xg(i), y, g.zmp[k]) >= 1e-10) {
                    if (c.ich == 1) val = 1.5 * c.udrv_i * (1.0 - y * y);
                    else if (c.ich == 2) val = (1.5 * (1.0 - y * y)) * 12.0;
                    else val = c.udrv_i;
                }
                s.u[g.ix(i, j, k)] = val;
            }
    for (int64_t k = 0; k <= g.n3; k++)
        for (int64_t i = 1; i <= g.n1; i++) {
            if (c.bc_ybtm == 0) { s.u[g.ix(i, 0, k)] = 0; s.u[g.ix(i, 1, k)] = 0; }
        }
    for (int64_t k = 0; k <= g.n3; k++)
        for (int64_t i = 1; i <= g.n1; i++) {
            if (c.bc_ytop == 0) { s.u[g.ix(i, g.n2m, k)] = 0; s.u[g.ix(i, g.n2, k)] = 0; }
        }
    for (int64_t j = 0; j <= g.n2; j++)
        for (int64_t i = 1; i <= g.n1; i++) {
            if (c.bc_zbtm == 0) { s.u[g.ix(i, j, 0)] = 0; s.u[g.ix(i, j, 1)] = 0; }
        }
    for (int64_t j = 0; j <= g.n2; j++)
        for (int64_t i = 1; i <= g.n1; i++) {
            if (c.bc_ztop == 0) { s.u[g.ix(i, j, g.n3m)] = 0; s.u[g.ix(i, j, g.n3)] = 0; }
        }
    if (c.ihtrans != 1) return s;
    for (int64_t k = 0; k <= g.n3; k++)
        for (int64_t j = 1; j <= g.n2m; j++)
            for (int64_t i = 0; i <= g.n1; i++)
                if (funcbody(c.body, g.xmp[i], g.ymp[j], g.zmp[k]) >= 1e-10) {
                    const double uu = s.u[g.ix(i, j, k)];
                    s.t[g.ix(i, j, k)] = c.idecomp == 1 ? (fabs(c.pr) > 1e-12 ? uu / c.pr : uu) : c.tflu_i;
                }
    if (c.xprdic == 0)
        for (int64_t k = 0; k <= g.n3; k++)
            for (int64_t j = 0; j <= g.n2; j++)
                s.t[g.ix(0, j, k)] = funcbody(c.body, g.xmp[0], g.ymp[j], g.zmp[k]) >= 1e-10 ? c.tflu_i : c.tsol_i;
    if (c.yprdic == 0)
        for (int64_t k = 0; k <= g.n3; k++)
            for (int64_t i = 0; i <= g.n1; i++) {
                if (c.bc_t_ybtm == 0) s.t[g.ix(i, 0, k)] = c.val_t_ybtm;
                else if (c.bc_t_ybtm == 1) s.t[g.ix(i, 0, k)] = s.t[g.ix(i, 1, k)] - c.val_t_ybtm / g.c2ci[1][1];
                if (c.bc_t_ytop == 0) s.t[g.ix(i, g.n2, k)] = c.val_t_ytop;
                else if (c.bc_t_ytop == 1)
                    s.t[g.ix(i, g.n2, k)] = s.t[g.ix(i, g.n2m, k)] + c.val_t_ytop / g.c2ci[1][g.n2];
            }
    if (c.zprdic == 0)
        for (int64_t j = 0; j <= g.n2; j++)
            for (int64_t i = 0; i <= g.n1; i++) {
                if (c.bc_t_zbtm == 0) s.t[g.ix(i, j, 0)] = c.val_t_zbtm;
                else if (c.bc_t_zbtm == 1) s.t[g.ix(i, j, 0)] = s.t[g.ix(i, j, 1)] - c.val_t_zbtm / g.c2ci[2][1];
                if (c.bc_t_ztop == 0) s.t[g.ix(i, j, g.n3)] = c.val_t_ztop;
                else if (c.bc_t_ztop == 1)
                    s.t[g.ix(i, j, g.n3)] = s.t[g.ix(i, j, g.n3m)] + c.val_t_ztop / g.c2ci[2][g.n3];
            }
    return s;
}

void writefield(const lesgpu_config &c, const Grid &g, const State &s, int64_t ihist) {
    char name[64];
    snprintf(name, sizeof(name), "../output/field/fld%07lld", (long long)ihist);
    std::vector<std::vector<char>> recs(9 + (c.ihtrans == 1 ? 1 : 0));
    put<int64_t>(recs[0], g.n1); put<int64_t>(recs[0], g.n2); put<int64_t>(recs[0], g.n3);
    put<double>(recs[0], c.re); put<double>(recs[0], c.pr); put<double>(recs[0], c.gr);
    put<int64_t>(recs[1], ihist); put<int64_t>(recs[1], s.m); put<double>(recs[1], s.time); put<double>(recs[1], s.dt);
    put<int64_t>(recs[2], c.xprdic); put<int64_t>(recs[2], c.yprdic); put<int64_t>(recs[2], c.zprdic);
    put<int64_t>(recs[3], c.xprdic == 1 ? 4 : 2); put<int64_t>(recs[3], c.xprdic == 1 ? 4 : 3);
    put<int64_t>(recs[3], c.bc_ybtm); put<int64_t>(recs[3], c.bc_ytop);
    put<int64_t>(recs[3], c.bc_zbtm); put<int64_t>(recs[3], c.bc_ztop);
    put<int64_t>(recs[4], c.ich); put<int64_t>(recs[4], c.iconjg);
    auto dump = [&](std::vector<char> &r, const std::vector<double> &a, int64_t i0, int64_t i1, int64_t j0, int64_t j1,
                    int64_t k0, int64_t k1) {
        for (int64_t k = k0; k <= k1; k++)
            for (int64_t j = j0; j <= j1; j++)
                for (int64_t i = i0; i <= i1; i++) put<double>(r, a[g.ix(i, j, k)]);
    };
    dump(recs[5], s.u, 1, g.n1, 0, g.n2, 0, g.n3);
    dump(recs[6], s.v, 0, g.n1, 1, g.n2, 0, g.n3);
    dump(recs[7], s.w, 0, g.n1, 0, g.n2, 1, g.n3);
    dump(recs[8], s.p, 1, g.n1m, 1, g.n2m, 1, g.n3m);
    if (c.ihtrans == 1) dump(recs[9], s.t, 1, g.n1m, 1, g.n2m, 1, g.n3m);
    write_records(name, recs);
}


// One field_avg file (misc_hist.f90:484-505): header records, then uavg vavg
// wavg uiujavg(6) pavg p2avg voravg(3) vor2avg(6) ssavg [tavg t2avg], each
// (n1m, n2m, n3m) in Fortran order; the name goes to fav_manifest.dat.
const int kFavGroups[11] = {1, 1, 1, 6, 1, 1, 3, 6, 1, 1, 1};

void write_fav(const lesgpu_config &c, const Grid &g, const std::vector<double> &a, double t0, double t1, int64_t h0,
               int64_t h1, bool combined) {
    const size_t ncell = (size_t)g.n1m * g.n2m * g.n3m;
    char name[64];
    snprintf(name, sizeof(name), "fav%07lld-%07lld", (long long)h0, (long long)h1);
    std::vector<std::vector<char>> recs(2);
    put<int64_t>(recs[0], g.n1m); put<int64_t>(recs[0], g.n2m); put<int64_t>(recs[0], g.n3m);
    put<double>(recs[0], c.re);
    put<double>(recs[1], t0); put<double>(recs[1], t1); put<double>(recs[1], (double)h0); put<double>(recs[1], (double)h1);
    const int ng = c.ihtrans == 1 ? 11 : 9;
    size_t a0 = 0;
    for (int q = 0; q < ng; q++) {
        std::vector<char> r(kFavGroups[q] * ncell * 8);
        memcpy(r.data(), a.data() + a0 * ncell, r.size());
        a0 += kFavGroups[q];
        recs.push_back(std::move(r));
    }
    const std::string dir = combined ? "../output/field_avg/combined/" : "../output/field_avg/";
    write_records(dir + name, recs);
    if (!combined) {
        FILE *mf = fopen("../output/field_avg/fav_manifest.dat", "a");
        if (mf) { fprintf(mf, "%s\n", name); fclose(mf); }
    }
}

// field_avg_finalize's combination (misc_hist.f90:608-700): the sums of all
// files named in fav_manifest.dat, with the first file's start and the last
// file's end, into field_avg/combined/.
void combine_favs(const lesgpu_config &c, const Grid &g) {
    std::ifstream man("../output/field_avg/fav_manifest.dat");
    if (!man) return;
    const size_t ncell = (size_t)g.n1m * g.n2m * g.n3m;
    const int ng = c.ihtrans == 1 ? 11 : 9;
    size_t nval = 0;
    for (int q = 0; q < ng; q++) nval += kFavGroups[q];
    std::vector<double> sum(nval * ncell, 0.0);
    double t0 = c.avg_tst, t1 = c.avg_tst;
    int64_t h0 = 0, h1 = 0, files = 0;
    std::string line;
    while (std::getline(man, line)) {
        while (!line.empty() && (line.back() == ' ' || line.back() == '\r')) line.pop_back();
        if (line.empty() || !exists("../output/field_avg/" + line)) continue;
        auto r = read_records("../output/field_avg/" + line);
        if (r.size() < 2 + (size_t)ng) continue;
        size_t pos = 0;
        double a0 = get<double>(r[1], pos), a1 = get<double>(r[1], pos);
        double b0 = get<double>(r[1], pos), b1 = get<double>(r[1], pos);
        size_t off = 0;
        for (int q = 0; q < ng; q++) {
            const size_t n = kFavGroups[q] * ncell;
            if (r[2 + q].size() != n * 8) die(line + ": record size does not match the grid");
            for (size_t z = 0; z < n; z++) {
                double v;
                memcpy(&v, r[2 + q].data() + 8 * z, 8);
                sum[off + z] += v;
            }
            off += n;
        }
        if (files == 0) { t0 = a0; h0 = llround(b0); }
        t1 = a1;
        h1 = llround(b1);
        files++;
    }
    if (files == 0) return;
    mkdir("../output/field_avg/combined", 0755);
    write_fav(c, g, sum, t0, t1, h0, h1, true);
}

// settings.input's tracking points (readsettings, misc_init.f90:53-59)
struct Trace {
    int64_t ntrace = 0, ntr = 0;
    std::vector<int64_t> pts;   // i, j, k of each point
};

// --dry-run: every value the readers produced, one "name value" per line
// (integers as integers, reals with 17 significant digits, arrays as their
// length and plain sum).
void dump_inputs(const lesgpu_config &c, const Grid &g, const Tables &t, const State &s, const Trace &tr,
                 const std::string &gridfile, const std::string &prev_fld) {
#define I_(f) printf(#f " %lld\n", (long long)c.f)
#define D_(f) printf(#f " %.17g\n", c.f)
    D_(re); D_(pr); D_(gr); I_(grdir); D_(tflu_i); D_(tsol_i);
    I_(ireset); I_(iread); I_(iavg); I_(ipzero); D_(eps_ptr); D_(udrv_i);
    I_(nend); I_(nprint); I_(npriavg); I_(npin); D_(tend); D_(ptb_tst); D_(avg_tst);
    I_(idtopt); D_(dt_size); D_(cflfac); D_(resid1); I_(nlev); I_(nbli); I_(ioldv); I_(mgitr); I_(imgsor); D_(wwsor);
    I_(iles); I_(insmdl); I_(itemdl); I_(idvmon); D_(csgsts); D_(csgshf); I_(filter);
    I_(ibmon); I_(masson); I_(imovingon); I_(ihtrans); I_(idecomp);
    I_(bc_ybtm); I_(bc_ytop); I_(bc_zbtm); I_(bc_ztop); I_(bc_t_ybtm); I_(bc_t_ytop); D_(val_t_ybtm); D_(val_t_ytop);
    I_(bc_t_zbtm); I_(bc_t_ztop); D_(val_t_zbtm); D_(val_t_ztop); I_(ich); I_(iconjg);
    I_(xprdic); I_(yprdic); I_(zprdic); I_(iintp); I_(poisson); I_(precision);
    I_(body.kind); D_(body.cx); D_(body.cy); D_(body.cz); D_(body.r); D_(body.p0);
#undef I_
#undef D_
    printf("grid %lld %lld %lld %lld %lld %lld\n", (long long)g.n1, (long long)g.n2, (long long)g.n3, (long long)g.n1m,
           (long long)g.n2m, (long long)g.n3m);
    auto dsum = [](const std::vector<double> &a) { double q = 0; for (double v : a) q += v; return q; };
    auto isum = [](const std::vector<int64_t> &a) { long long q = 0; for (int64_t v : a) q += v; return q; };
    printf("x %zu %.17g\nymp %zu %.17g\nc2cy %zu %.17g\n", g.x.size(), dsum(g.x), g.ymp.size(), dsum(g.ymp),
           g.c2c[1].size(), dsum(g.c2c[1]));
    for (int l = 0; l < 4; l++)
        printf("ibm%d %lld %lld %lld %lld %.17g\n", l, (long long)t.nintp[l], (long long)t.nbody[l], isum(t.fc[l]),
               isum(t.ix[l]), dsum(t.gf[l]));
    printf("nzero %lld %lld %lld %lld\n", (long long)t.nzero, isum(t.inz), isum(t.jnz), isum(t.knz));
    printf("nwall %zu %lld\ncstar %zu %.17g\nkstar %zu %.17g\n", t.nwall.size(), isum(t.nwall), t.cstar.size(),
           dsum(t.cstar), t.kstar.size(), dsum(t.kstar));
    printf("state %lld %lld %.17g %.17g\n", (long long)s.ihist, (long long)s.m, s.time, s.dt);
    printf("gridfile %s\nprev_fld %s\n", gridfile.c_str(), prev_fld.c_str());
    printf("trace %lld %lld", (long long)tr.ntrace, (long long)tr.ntr);
    for (int64_t v : tr.pts) printf(" %lld", (long long)v);
    printf("\n");
    printf("fields %.17g %.17g %.17g %.17g %.17g\n", dsum(s.u), dsum(s.v), dsum(s.w), dsum(s.p), dsum(s.t));
}

}  // namespace

int main(int argc, char **argv) {
    int device = 0;
    bool dry_run = false;
    for (int a = 1; a < argc; a++) {
        if (!strcmp(argv[a], "--device") && a + 1 < argc) device = atoi(argv[++a]);
        else if (!strcmp(argv[a], "--dry-run")) dry_run = true;
        else die(std::string("usage: lesgpu_exec [--device N] [--dry-run]; unknown option ") + argv[a]);
    }
    if (!dry_run)
        for (const char *d : {"../output", "../output/field", "../output/ftr", "../output/field_avg"}) mkdir(d, 0755);

    // ---- readsettings, misc_init.f90:19-92
    lesgpu_config c;
    memset(&c, 0, sizeof(c));
    std::string gridfile, prev_fld;
    Trace trace;
    {
        ListReader r("settings.input");
        r.skip();
        auto v = r.items(6);
        c.re = to_d(v[0]); c.pr = to_d(v[1]); c.gr = to_d(v[2]); c.grdir = to_i(v[3]); c.tflu_i = to_d(v[4]); c.tsol_i = to_d(v[5]);
        r.skip();
        v = r.items(6);
        c.ireset = to_i(v[0]); c.iread = to_i(v[1]); c.iavg = to_i(v[2]); c.ipzero = to_i(v[3]); c.eps_ptr = to_d(v[4]); c.udrv_i = to_d(v[5]);
        r.skip();
        v = r.items(4);
        c.nend = to_i(v[0]); c.nprint = to_i(v[1]); c.npriavg = to_i(v[2]); c.npin = to_i(v[3]);
        r.skip();
        v = r.items(3);
        c.tend = to_d(v[0]); c.ptb_tst = to_d(v[1]); c.avg_tst = to_d(v[2]);
        r.skip();
        v = r.items(3);
        c.idtopt = to_i(v[0]); c.dt_size = to_d(v[1]); c.cflfac = to_d(v[2]);
        r.skip();
        v = r.items(7);
        c.resid1 = to_d(v[0]); c.nlev = to_i(v[1]); c.nbli = to_i(v[2]); c.ioldv = to_i(v[3]); c.mgitr = to_i(v[4]);
        c.imgsor = to_i(v[5]); c.wwsor = to_d(v[6]);
        r.skip();
        v = r.items(7);
        c.iles = to_i(v[0]); c.insmdl = to_i(v[1]); c.itemdl = to_i(v[2]); c.idvmon = to_i(v[3]); c.csgsts = to_d(v[4]);
        c.csgshf = to_d(v[5]); c.filter = to_i(v[6]);
        r.skip();
        v = r.items(5);
        c.ibmon = to_i(v[0]); c.masson = to_i(v[1]); c.imovingon = to_i(v[2]); c.ihtrans = to_i(v[3]); c.idecomp = to_i(v[4]);
        r.skip();
        gridfile = r.items(1)[0];
        prev_fld = r.items(1)[0];
        // TRACE NTR and the tracking points (the tracer histories themselves
        // are not written); rows after the last point are not read
        r.skip();
        v = r.items(2);
        trace.ntrace = to_i(v[0]);
        trace.ntr = to_i(v[1]);
        for (int64_t n = 0; n < trace.ntrace; n++) {
            v = r.items(3);
            for (int q = 0; q < 3; q++) trace.pts.push_back(to_i(v[q]));
        }
    }
    // ---- readbcs, misc_init.f90:95-158
    {
        ListReader r("boundary.input");
        r.skip();
        auto v = r.items(2); c.bc_ybtm = to_i(v[0]); c.bc_ytop = to_i(v[1]);
        r.skip();
        v = r.items(2); c.bc_zbtm = to_i(v[0]); c.bc_ztop = to_i(v[1]);
        r.skip();
        v = r.items(2); c.bc_t_ybtm = to_i(v[0]); c.bc_t_ytop = to_i(v[1]);
        r.skip();
        v = r.items(2); c.val_t_ybtm = to_d(v[0]); c.val_t_ytop = to_d(v[1]);
        r.skip();
        v = r.items(2); c.bc_t_zbtm = to_i(v[0]); c.bc_t_ztop = to_i(v[1]);
        r.skip();
        v = r.items(2); c.val_t_zbtm = to_d(v[0]); c.val_t_ztop = to_d(v[1]);
        r.skip();
        v = r.items(2); c.ich = to_i(v[0]); c.iconjg = to_i(v[1]);
        ListReader q("../output/ibmpre/ibmpre_prdic.bin");
        v = q.items(4);
        c.xprdic = to_i(v[0]); c.yprdic = to_i(v[1]); c.zprdic = to_i(v[2]); c.iintp = to_i(v[3]);
        if (c.yprdic == 1) c.bc_ybtm = c.bc_ytop = 4;
        if (c.zprdic == 1) c.bc_zbtm = c.bc_ztop = 4;
    }
    // ---- body, Poisson solver and arithmetic form (compile-time in the reference)
    {
        ListReader r("body.input");
        r.skip();
        auto v = r.items(8);
        c.body.kind = to_i(v[0]); c.body.cx = to_d(v[1]); c.body.cy = to_d(v[2]); c.body.cz = to_d(v[3]);
        c.body.r = to_d(v[4]); c.body.p0 = to_d(v[5]);
        c.poisson = to_i(v[6]); c.precision = to_i(v[7]);
    }
    // ---- readgeom, tables, field
    Grid g = readgeom(gridfile);
    Tables t;
    if (c.ibmon == 1) t = read_tables(c, g);
    State s;
    if (c.iread == 1) {
        s = prefld(prev_fld, c, g);
    } else {
        if (c.eps_ptr != 0.0) fprintf(stderr, "lesgpu_exec: EPS_PTR perturbation is not applied\n");
        s = makefld(c, g);
        if (!dry_run) writefield(c, g, s, 0);
    }
    if (c.ireset == 1) { s.ihist = 0; s.time = 0.0; }
    if (dry_run) {            // what was read, for checking the readers without a GPU
        dump_inputs(c, g, t, s, trace, gridfile, prev_fld);
        return 0;
    }
    check(lesgpu_set_device(device), "set_device");
    if (c.iavg == 1 && c.iread != 1) {                 // dttimeinit empties the manifest
        FILE *mf = fopen("../output/field_avg/fav_manifest.dat", "w");
        if (mf) fclose(mf);
    }

    lesgpu_grid lg_;
    memset(&lg_, 0, sizeof(lg_));
    lg_.n1 = g.n1; lg_.n2 = g.n2; lg_.n3 = g.n3; lg_.n1m = g.n1m; lg_.n2m = g.n2m; lg_.n3m = g.n3m;
    lg_.xl = g.xl; lg_.yl = g.yl; lg_.zl = g.zl;
    lg_.x = g.x.data(); lg_.y = g.y.data(); lg_.z = g.z.data();
    lg_.ipv = g.pv[0].data(); lg_.jpv = g.pv[1].data(); lg_.kpv = g.pv[2].data();
    lg_.imv = g.mv[0].data(); lg_.jmv = g.mv[1].data(); lg_.kmv = g.mv[2].data();
    lg_.fixil = g.fl[0].data(); lg_.fixjl = g.fl[1].data(); lg_.fixkl = g.fl[2].data();
    lg_.fixiu = g.fu[0].data(); lg_.fixju = g.fu[1].data(); lg_.fixku = g.fu[2].data();
    lg_.c2cx = g.c2c[0].data(); lg_.c2cy = g.c2c[1].data(); lg_.c2cz = g.c2c[2].data();
    lg_.c2cxi = g.c2ci[0].data(); lg_.c2cyi = g.c2ci[1].data(); lg_.c2czi = g.c2ci[2].data();
    lg_.f2fx = g.f2f[0].data(); lg_.f2fy = g.f2f[1].data(); lg_.f2fz = g.f2f[2].data();
    lg_.f2fxi = g.f2fi[0].data(); lg_.f2fyi = g.f2fi[1].data(); lg_.f2fzi = g.f2fi[2].data();
    lg_.xmp = g.xmp.data(); lg_.ymp = g.ymp.data(); lg_.zmp = g.zmp.data();

    lesgpu_case *cs = nullptr;
    check(lesgpu_create(&c, &lg_, &cs), "create");
    lesgpu_ibm b;
    memset(&b, 0, sizeof(b));
    for (int l = 0; l < 4; l++) {
        b.nintp[l] = t.nintp[l]; b.nbody[l] = t.nbody[l];
        b.fc[l] = t.fc[l].empty() ? nullptr : t.fc[l].data();
        b.intpindx[l] = t.ix[l].empty() ? nullptr : t.ix[l].data();
        b.geomfac[l] = t.gf[l].empty() ? nullptr : t.gf[l].data();
    }
    b.nzero = t.nzero;
    b.inz = t.inz.empty() ? nullptr : t.inz.data();
    b.jnz = t.jnz.empty() ? nullptr : t.jnz.data();
    b.knz = t.knz.empty() ? nullptr : t.knz.data();
    b.nwall_dvm = t.nwall.empty() ? nullptr : t.nwall.data();
    b.cstar = t.cstar.empty() ? nullptr : t.cstar.data();
    b.kstar = t.kstar.empty() ? nullptr : t.kstar.data();
    b.omega = t.omega.empty() ? nullptr : t.omega.data();
    check(lesgpu_load_ibm(cs, &b), "load_ibm");
    check(lesgpu_set_fields(cs, s.u.data(), s.v.data(), s.w.data(), s.p.data(), s.t.data(), s.time, s.dt, s.ihist, s.m),
          "set_fields");
    check(lesgpu_start(cs), "start");

    // ---- history files (ftrfiles, misc_hist.f90:1-62)
    const char *mode = c.iread == 1 ? "a" : "w";
    FILE *fhist = fopen("../output/ftr/fhist.dat", mode), *fcd = fopen("../output/ftr/fcdcl.dat", mode);
    FILE *fhf = fopen("../output/ftr/fheatflux.dat", mode), *ftemp = fopen("../output/ftr/ftemp.dat", mode);
    FILE *fcmfr = c.ich != 0 ? fopen("../output/ftr/fcmfr.dat", mode) : nullptr;
    FILE *ftime = fopen("../output/ftr/ftime.dat", mode);
    if (!fhist || !fcd || !fhf || !ftemp || !ftime || (c.ich != 0 && !fcmfr)) die("cannot open ../output/ftr/*.dat");

    // volume of the fluid u cells (writehistory's flowvol; the body is stationary)
    double flowvol = 0.0;
    for (int64_t k = 1; k <= g.n3m; k++)
        for (int64_t j = 1; j <= g.n2m; j++)
            for (int64_t i = 1; i <= g.n1m; i++)
                if (funcbody(c.body, g.x[i - 1], g.ymp[j], g.zmp[k]) >= 1e-10)
                    flowvol += g.c2c[0][i] * g.f2f[1][j] * g.f2f[2][k];
    double cmfr_int[3] = {0, 0, 0}, cmfr_dur = 0, tb_int[2] = {0, 0}, tb_dur = 0;
    double cd_int[3] = {0, 0, 0}, cd_dur = 0, hf_int[3] = {0, 0, 0}, hf_dur = 0;
    int64_t ntime = 0, ihist = s.ihist;
    double time = s.time;
    int64_t avg_nsamples = 0, ihistinit = ihist;
    double timeinit = c.avg_tst;
    bool avg_started = false;
    const int navg = c.ihtrans == 1 ? LESGPU_NAVG : LESGPU_NAVG - 2;
    const size_t ncell = (size_t)g.n1m * g.n2m * g.n3m;
    lesgpu_step_report rep;

    // ---- the time loop, solver.f90:85-183
    while (ntime < c.nend && time < c.tend) {
        check(lesgpu_step(cs, &rep), "step");
        // the reference's multigrid prints this once per mode that reached
        // MGITR (poiss_z_ft.f90:289) and carries on
        for (int64_t q = 0; q < rep.poisson_unconverged; q++) printf(" ITERATION LIMIT EXCEEDED.\n");
        ntime = rep.ntime;
        time = rep.time;
        const double dt = rep.dt;
        if (ntime % c.npin == 0) {                                  // writehistory
            ihist += 1;
            fprintf(fhist, "%13.5f%15.7E%15.7E%15.7E%15.7E\n", time, dt, rep.cflmax, rep.dvmax, rep.qmmax);
            if (c.ich != 0) {
                const double qflux = rep.qflux;
                double avg[3] = {0, 0, 0};
                if (time >= c.avg_tst) {
                    cmfr_int[0] += qflux * dt; cmfr_int[1] += rep.ubulk * dt; cmfr_int[2] += rep.pmiavg * dt;
                    cmfr_dur += dt;
                    for (int q = 0; q < 3; q++) avg[q] = cmfr_int[q] / cmfr_dur;
                }
                fprintf(fcmfr, "%13.5f%15.7E%15.7E%15.7E%15.7E%15.7E%15.7E\n", time, qflux, rep.ubulk, rep.pmiavg,
                        avg[0], avg[1], avg[2]);
            }
            if (c.ihtrans == 1) {
                double avg[2] = {0, 0};
                if (time >= c.avg_tst) {
                    tb_int[0] += rep.tbulk_fluid * dt; tb_int[1] += rep.tbulk_solid * dt; tb_dur += dt;
                    avg[0] = tb_int[0] / tb_dur; avg[1] = tb_int[1] / tb_dur;
                }
                fprintf(ftemp, "%13.5f%15.7E%15.7E%15.7E%15.7E\n", time, rep.tbulk_fluid, rep.tbulk_solid, avg[0], avg[1]);
            }
        }
        if (c.ibmon == 1) {                                        // draglift's history
            double avg[3] = {0, 0, 0};
            if (time >= c.avg_tst) {
                for (int q = 0; q < 3; q++) cd_int[q] += rep.cd[q] * dt;
                cd_dur += dt;
                for (int q = 0; q < 3; q++) avg[q] = cd_int[q] / cd_dur;
            }
            if (ntime % c.npin == 0)
                fprintf(fcd, "%13.5f%15.7E%15.7E%15.7E%15.7E%15.7E%15.7E\n", time, rep.cd[0], rep.cd[1], rep.cd[2],
                        avg[0], avg[1], avg[2]);
        }
        if (c.ihtrans == 1) {                                      // heatflux's history
            double avg[3] = {0, 0, 0};
            if (time >= c.avg_tst) {
                for (int q = 0; q < 3; q++) hf_int[q] += rep.heat_flux[q] * dt;
                hf_dur += dt;
                for (int q = 0; q < 3; q++) avg[q] = hf_int[q] / hf_dur;
            }
            if (ntime % c.npin == 0)
                fprintf(fhf, "%13.5f%15.7E%15.7E%15.7E%15.7E%15.7E%15.7E\n", time, rep.heat_flux[0], rep.heat_flux[1],
                        rep.heat_flux[2], avg[0], avg[1], avg[2]);
        }
        if (ntime % c.nprint == 0) {                                // writefield
            check(lesgpu_get_fields(cs, s.u.data(), s.v.data(), s.w.data(), s.p.data(), s.t.data()), "get_fields");
            s.m = rep.m; s.time = time; s.dt = dt;
            writefield(c, g, s, ihist);
        }
        if (c.iavg == 1 && time > c.avg_tst) {                      // field_avg's file every NPRIAVG samples
            if (!avg_started) { avg_started = true; ihistinit = ihist; timeinit = c.avg_tst; }
            if (++avg_nsamples >= c.npriavg) {
                std::vector<double> a((size_t)navg * ncell);
                int64_t ns = 0;
                check(lesgpu_get_averages(cs, a.data(), &ns, 1), "get_averages");
                write_fav(c, g, a, timeinit, time, ihistinit, ihist, false);
                avg_nsamples = 0;
                ihistinit = ihist;
                timeinit = time;
            }
        }
        // writeftrtime, misc_hist.f90:255-282 (device time of each phase group)
        printf("TIME FOR SGS    : %12.3f SECONDS\nTIME FOR RHSNLHS: %12.3f SECONDS\n"
               "TIME FOR POISSON: %12.3f SECONDS\nTIME OF OPERTION: %12.3f SECONDS\n",
               rep.phase_ms[0] * 1e-3, rep.phase_ms[1] * 1e-3, rep.phase_ms[2] * 1e-3, rep.phase_ms[3] * 1e-3);
        fprintf(ftime, "%13.5f%15.7E%15.7E%15.7E%15.7E\n", time, rep.phase_ms[0] * 1e-3, rep.phase_ms[1] * 1e-3,
                rep.phase_ms[2] * 1e-3, rep.phase_ms[3] * 1e-3);
    }
    // ---- finish, solver.f90:188-191
    if (ntime % c.nprint != 0) {
        check(lesgpu_get_fields(cs, s.u.data(), s.v.data(), s.w.data(), s.p.data(), s.t.data()), "get_fields");
        s.m = rep.m; s.time = time; s.dt = rep.dt;
        writefield(c, g, s, ihist);
    }
    if (c.iavg == 1 && avg_started) {                               // field_avg_finalize
        if (avg_nsamples > 0) {
            std::vector<double> a((size_t)navg * ncell);
            int64_t ns = 0;
            check(lesgpu_get_averages(cs, a.data(), &ns, 1), "get_averages");
            write_fav(c, g, a, timeinit, time, ihistinit, ihist, false);
        }
        combine_favs(c, g);
    }
    for (FILE *f : {fhist, fcd, fhf, ftemp, ftime}) fclose(f);
    if (fcmfr) fclose(fcmfr);
    check(lesgpu_destroy(cs), "destroy");
    printf("lesgpu_exec: %lld steps, time %.6f, dvmax %.3e\n", (long long)ntime, time, rep.dvmax);
    return 0;
}
