// io.cpp -- the reference's input_parameters reader (input_output.f90:21-133)
// and its big-endian stream snapshot format (input_output.f90:231-544).
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>

#include <cmath>
#include <fstream>
#include <sstream>
#include <string>
#include <vector>

#include "channel_gpu.h"

namespace {

// Fortran list-directed input, one READ per call: values are taken from the
// current record and, if it runs short, from the following records; the READ
// then leaves the rest of its last record unread (the next READ starts on a
// new record).
struct ListReader {
    std::vector<std::string> lines;
    size_t cur = 0;

    static void tokenize(const std::string &l, std::vector<std::string> &out) {
        size_t i = 0, n = l.size();
        while (i < n) {
            while (i < n && (l[i] == ' ' || l[i] == '\t' || l[i] == ',' || l[i] == '\r')) i++;
            if (i >= n) break;
            if (l[i] == '\'' || l[i] == '"') {
                char q = l[i++];
                std::string s;
                while (i < n && l[i] != q) s += l[i++];
                i++;
                out.push_back(s);
            } else {
                std::string s;
                while (i < n && l[i] != ' ' && l[i] != '\t' && l[i] != ',' && l[i] != '\r') s += l[i++];
                out.push_back(s);
            }
        }
    }
    bool read(int nvals, std::vector<std::string> &vals) {
        vals.clear();
        while ((int)vals.size() < nvals) {
            if (cur >= lines.size()) return false;
            std::vector<std::string> t;
            tokenize(lines[cur++], t);
            for (auto &s : t)
                if ((int)vals.size() < nvals) vals.push_back(s);
        }
        return true;
    }
    bool skip() {
        if (cur >= lines.size()) return false;
        cur++;
        return true;
    }
};

bool to_double(const std::string &s, double &v) {
    std::string t = s;
    for (auto &c : t)
        if (c == 'd' || c == 'D') c = 'e';
    char *end = nullptr;
    v = strtod(t.c_str(), &end);
    return end && *end == 0 && !t.empty();
}
bool to_int(const std::string &s, int &v) {
    char *end = nullptr;
    long l = strtol(s.c_str(), &end, 10);
    v = (int)l;
    return end && *end == 0 && !s.empty();
}

inline uint32_t bswap32(uint32_t x) {
    return ((x & 0xffu) << 24) | ((x & 0xff00u) << 8) | ((x >> 8) & 0xff00u) | (x >> 24);
}
inline uint64_t bswap64(uint64_t x) {
    return ((uint64_t)bswap32((uint32_t)(x & 0xffffffffu)) << 32) | bswap32((uint32_t)(x >> 32));
}
inline bool little_endian() {
    uint16_t one = 1;
    return *(const unsigned char *)&one == 1;
}

bool read_i32(FILE *f, int32_t &v) {
    uint32_t u;
    if (fread(&u, 4, 1, f) != 1) return false;
    if (little_endian()) u = bswap32(u);
    memcpy(&v, &u, 4);
    return true;
}
bool read_f64(FILE *f, double *v, size_t n) {
    std::vector<uint64_t> buf(n);
    if (n && fread(buf.data(), 8, n, f) != n) return false;
    for (size_t q = 0; q < n; q++) {
        uint64_t u = little_endian() ? bswap64(buf[q]) : buf[q];
        memcpy(&v[q], &u, 8);
    }
    return true;
}
bool write_i32(FILE *f, int32_t v) {
    uint32_t u;
    memcpy(&u, &v, 4);
    if (little_endian()) u = bswap32(u);
    return fwrite(&u, 4, 1, f) == 1;
}
bool write_f64(FILE *f, const double *v, size_t n) {
    std::vector<uint64_t> buf(n);
    for (size_t q = 0; q < n; q++) {
        uint64_t u;
        memcpy(&u, &v[q], 8);
        buf[q] = little_endian() ? bswap64(u) : u;
    }
    return n == 0 || fwrite(buf.data(), 8, n, f) == n;
}

}  // namespace

extern "C" int cf_read_input_parameters(const char *path, cf_params *p, int grid[3], char filein[200],
                                        char fileout[200], int ints[4], int ints2[2]) {
    if (!path || !p) return CF_ERR_INVALID;
    std::ifstream in(path);
    if (!in) return CF_ERR_IO;
    ListReader r;
    std::string line;
    while (std::getline(in, line)) r.lines.push_back(line);
    cf_default_params(p);
    std::vector<std::string> v;
    int g[3], iv[4], i2[2] = {0, 0}, gwm[3], ai[6], est;
    double dv[5];
    std::string fi, fo;
#define SKIP()                          \
    if (!r.skip()) return CF_ERR_INVALID
#define READ(n)                          \
    if (!r.read(n, v)) return CF_ERR_INVALID
#define INT(k, dst)                      \
    if (!to_int(v[k], dst)) return CF_ERR_INVALID
#define DBL(k, dst)                      \
    if (!to_double(v[k], dst)) return CF_ERR_INVALID
    SKIP(); READ(3); INT(0, g[0]); INT(1, g[1]); INT(2, g[2]);          // nx ny nz
    SKIP(); READ(1); DBL(0, p->CFL);                                    // CFL
    SKIP(); READ(2); INT(0, p->Retau_int); DBL(1, p->nu);               // Retau_int, nu
    SKIP(); READ(4); DBL(0, p->dPdx); DBL(1, p->dPdz); INT(2, p->x_mass_cte); INT(3, p->y_mass_cte);
    SKIP(); READ(1); INT(0, p->LES_model);
    SKIP(); READ(1); INT(0, p->iwall_model);
    SKIP(); READ(5); for (int q = 0; q < 5; q++) DBL(q, dv[q]);         // alphas, alpha_std, freq_mult
    p->freq_mult = dv[4];
    SKIP(); READ(4); for (int q = 0; q < 4; q++) INT(q, iv[q]);         // nsteps nsave nstats nmonitor
    SKIP(); READ(1); fi = v[0];
    SKIP(); READ(1); fo = v[0];
    SKIP(); READ(1); INT(0, i2[0]);                                     // nstep_init
    SKIP(); READ(1); INT(0, i2[1]);                                     // random_init
    SKIP(); READ(1); DBL(0, p->Rossby_plus);
    SKIP(); READ(1); INT(0, p->Dirichlet_nu_t);
    SKIP(); READ(2); INT(0, p->jref_eqwm); INT(1, est);
    SKIP(); READ(1); { double fs; DBL(0, fs); }                         // fil_size_2 (slip models only)
    SKIP(); SKIP(); READ(3); for (int q = 0; q < 3; q++) INT(q, gwm[q]);
    SKIP(); READ(6); for (int q = 0; q < 6; q++) INT(q, ai[q]);
#undef SKIP
#undef READ
#undef INT
#undef DBL
    if (grid) for (int q = 0; q < 3; q++) grid[q] = g[q];
    if (ints) for (int q = 0; q < 4; q++) ints[q] = iv[q];
    if (ints2) { ints2[0] = i2[0]; ints2[1] = i2[1]; }
    if (filein) { strncpy(filein, fi.c_str(), 199); filein[199] = 0; }
    if (fileout) { strncpy(fileout, fo.c_str(), 199); fileout[199] = 0; }
    return CF_OK;
}

extern "C" int cf_read_snapshot(const char *path, int nx, int ny, int nz, double *x, double *y, double *z, double *U,
                                double *V, double *W) {
    FILE *f = fopen(path, "rb");
    if (!f) return CF_ERR_IO;
    int rc = CF_OK;
    int32_t n;
    std::vector<double> tmp;
    const int nn[6] = {nx, ny, nz, nx - 1, ny - 1, nz - 1};
    double *dst[6] = {x, y, z, nullptr, nullptr, nullptr};
    for (int q = 0; q < 6 && rc == CF_OK; q++) {  // input_output.f90:244-266
        if (!read_i32(f, n) || n != nn[q]) { rc = CF_ERR_INVALID; break; }
        tmp.resize(n);
        if (!read_f64(f, tmp.data(), n)) { rc = CF_ERR_IO; break; }
        if (dst[q]) memcpy(dst[q], tmp.data(), n * sizeof(double));
    }
    const int shp[3][3] = {{nx, ny + 1, nz + 1}, {nx + 1, ny, nz + 1}, {nx + 1, ny + 1, nz}};
    double *fld[3] = {U, V, W};
    for (int q = 0; q < 3 && rc == CF_OK; q++) {  // input_output.f90:279-362
        int32_t s[3];
        if (!read_i32(f, s[0]) || !read_i32(f, s[1]) || !read_i32(f, s[2])) { rc = CF_ERR_IO; break; }
        if (s[0] != shp[q][0] || s[1] != shp[q][1] || s[2] != shp[q][2]) { rc = CF_ERR_INVALID; break; }
        size_t cnt = (size_t)s[0] * s[1] * s[2];
        if (fld[q]) {
            if (!read_f64(f, fld[q], cnt)) rc = CF_ERR_IO;
        } else if (fseek(f, (long)(cnt * 8), SEEK_CUR) != 0) {
            rc = CF_ERR_IO;
        }
    }
    fclose(f);
    return rc;
}

extern "C" int cf_write_snapshot(const char *path, int nx, int ny, int nz, const double *x, const double *y,
                                 const double *z, const double *U, const double *V, const double *W, const double *P,
                                 const double *nu_t) {
    FILE *f = fopen(path, "wb");
    if (!f) return CF_ERR_IO;
    bool ok = true;
    std::vector<double> xm(nx - 1), ym(ny - 1), zm(nz - 1);  // initialization.f90:169-177
    for (int i = 0; i < nx - 1; i++) xm[i] = 0.5 * (x[i] + x[i + 1]);
    for (int j = 0; j < ny - 1; j++) ym[j] = 0.5 * (y[j] + y[j + 1]);
    for (int k = 0; k < nz - 1; k++) zm[k] = 0.5 * (z[k] + z[k + 1]);
    const double *m[6] = {x, y, z, xm.data(), ym.data(), zm.data()};
    const int nn[6] = {nx, ny, nz, nx - 1, ny - 1, nz - 1};
    for (int q = 0; q < 6; q++) ok = ok && write_i32(f, nn[q]) && write_f64(f, m[q], nn[q]);  // :416-422
    const int shp[5][3] = {{nx, ny + 1, nz + 1}, {nx + 1, ny, nz + 1}, {nx + 1, ny + 1, nz}, {nx + 1, ny + 1, nz + 1},
                           {nx + 1, ny + 1, nz + 1}};
    const double *fld[5] = {U, V, W, P, nu_t};
    for (int q = 0; q < 5; q++) {  // :432-535
        if (!fld[q]) continue;
        ok = ok && write_i32(f, shp[q][0]) && write_i32(f, shp[q][1]) && write_i32(f, shp[q][2]);
        ok = ok && write_f64(f, fld[q], (size_t)shp[q][0] * shp[q][1] * shp[q][2]);
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? CF_OK : CF_ERR_IO;
}

// ---------------------------------------------------------------------------
// Statistics text file, output_statistics (input_output.f90:549-570).
// ---------------------------------------------------------------------------
namespace {

// Fortran Fw.d output of one REAL(8): correctly rounded fixed point, right
// justified; w asterisks when it does not fit (after dropping the optional
// leading zero).  IEEE -0.0 is written without sign (the default
// "nominus0" behaviour of the Intel compiler the reference targets); other
// negative values keep it, also when they round to zero.
std::string fortran_f(double v, int w, int d) {
    std::string s;
    if (std::isnan(v)) {
        s = "NaN";
    } else if (std::isinf(v)) {
        s = v > 0 ? (w >= 8 ? "Infinity" : "Inf") : (w >= 9 ? "-Infinity" : "-Inf");
    } else {
        char buf[400];
        snprintf(buf, sizeof buf, "%.*f", d, v == 0.0 ? 0.0 : v);
        s = buf;
        if ((int)s.size() > w) {
            if (s.compare(0, 2, "0.") == 0) s.erase(0, 1);
            else if (s.compare(0, 3, "-0.") == 0) s.erase(1, 1);
        }
    }
    if ((int)s.size() > w) return std::string((size_t)w, '*');
    return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

// Fortran Iw output
std::string fortran_i(long v, int w) {
    char buf[32];
    snprintf(buf, sizeof buf, "%ld", v);
    std::string s = buf;
    if ((int)s.size() > w) return std::string((size_t)w, '*');
    return std::string((size_t)(w - (int)s.size()), ' ') + s;
}

}  // namespace

extern "C" int cf_statistics_file_name(const char *fileout, int istep, int nstep_init, char *name, int cap) {
    if (!fileout || !name || cap <= 0) return CF_ERR_INVALID;
    // Trim(Adjustl(fileout)) // '.' // Trim(Adjustl(ext)) // '.stats.txt', ext written with I8
    std::string f = fileout;
    size_t a = f.find_first_not_of(' ');
    f = a == std::string::npos ? std::string() : f.substr(a);
    while (!f.empty() && f.back() == ' ') f.pop_back();
    std::string ext = fortran_i((long)istep + nstep_init, 8);
    ext.erase(0, ext.find_first_not_of(' '));
    std::string n = f + "." + ext + ".stats.txt";
    if ((int)n.size() + 1 > cap) return CF_ERR_INVALID;
    memcpy(name, n.c_str(), n.size() + 1);
    return CF_OK;
}

extern "C" int cf_write_statistics(const char *path, double t, double nu, int nx, int ny, int nz, int istep,
                                   const double *y, const double *stats) {
    if (!path || !y || !stats || ny < 1) return CF_ERR_INVALID;
    FILE *f = fopen(path, "w");
    if (!f) return CF_ERR_IO;
    const double *Um = stats, *U2 = stats + 3 * ny, *V2 = stats + 4 * ny, *W2 = stats + 5 * ny, *UV = stats + 6 * ny,
                 *P2 = stats + 8 * ny;
    const double utau = stats[9 * ny], Retau = stats[9 * ny + 1];
    // '(A,4F15.8,4I)': the Intel compiler's default width for an INTEGER(4)
    // I descriptor without width is 12
    std::string line = "%" + fortran_f(t, 15, 8) + fortran_f(Retau, 15, 8) + fortran_f(utau, 15, 8) +
                       fortran_f(nu, 15, 8) + fortran_i(nx, 12) + fortran_i(ny, 12) + fortran_i(nz, 12) +
                       fortran_i(istep, 12) + "\n";
    bool ok = fputs(line.c_str(), f) >= 0;
    for (int j = 0; j < ny && ok; j++) {  // '(8F15.8)' with seven items per record
        line = fortran_f(y[j], 15, 8) + fortran_f(Um[j], 15, 8) + fortran_f(U2[j], 15, 8) + fortran_f(V2[j], 15, 8) +
               fortran_f(W2[j], 15, 8) + fortran_f(UV[j], 15, 8) + fortran_f(P2[j], 15, 8) + "\n";
        ok = fputs(line.c_str(), f) >= 0;
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? CF_OK : CF_ERR_IO;
}
