// fm3dt_files.cpp -- readers and writers of the reference program's files.
#include "fm3dt_files.h"

#include <cerrno>
#include <cmath>
#include <cstdlib>
#include <cstring>

namespace fm3dt_io {

namespace {

std::string trim(const std::string &s)
{
    size_t a = 0, b = s.size();
    while (a < b && (s[a] == ' ' || s[a] == '\t' || s[a] == '\r')) ++a;
    while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r')) --b;
    return s.substr(a, b - a);
}

// (a20): the first 20 characters of the record; OPEN ignores the trailing
// blanks of a file name.
std::string a20(const std::string &line) { return trim(line.substr(0, line.size() < 20 ? line.size() : 20)); }

bool parse_double(const std::string &tok, double &v)
{
    std::string t = tok;
    for (char &c : t)
        if (c == 'd' || c == 'D') c = 'e';
    errno = 0;
    char *end = nullptr;
    v = std::strtod(t.c_str(), &end);
    return errno == 0 && end && *end == '\0' && !t.empty();
}

bool parse_float(const std::string &tok, float &v)
{
    std::string t = tok;
    for (char &c : t)
        if (c == 'd' || c == 'D') c = 'e';
    errno = 0;
    char *end = nullptr;
    v = std::strtof(t.c_str(), &end);
    return errno == 0 && end && *end == '\0' && !t.empty();
}

bool parse_int(const std::string &tok, int &v)
{
    errno = 0;
    char *end = nullptr;
    const long x = std::strtol(tok.c_str(), &end, 10);
    if (errno || !end || *end != '\0' || tok.empty() || x < -2147483647L - 1 || x > 2147483647L) return false;
    v = (int)x;
    return true;
}

}  // namespace

ListReader::ListReader(const std::string &path) { f_ = std::fopen(path.c_str(), "rb"); }

ListReader::~ListReader()
{
    if (f_) std::fclose(f_);
}

bool ListReader::record(std::string &line)
{
    line.clear();
    if (!f_) return false;
    int c;
    bool any = false;
    while ((c = std::fgetc(f_)) != EOF) {
        any = true;
        if (c == '\n') break;
        line.push_back((char)c);
    }
    if (!any) return false;
    if (!line.empty() && line.back() == '\r') line.pop_back();
    ++line_no_;
    return true;
}

bool ListReader::tokens(std::vector<std::string> &out, int n)
{
    out.clear();
    std::string line;
    while ((int)out.size() < n) {
        if (!record(line)) return false;
        size_t i = 0;
        bool stop = false;
        while (i < line.size() && (int)out.size() < n && !stop) {
            while (i < line.size() && (line[i] == ' ' || line[i] == '\t' || line[i] == ',')) ++i;
            if (i >= line.size()) break;
            if (line[i] == '/') { stop = true; break; }   // slash ends the read
            size_t j = i;
            while (j < line.size() && line[j] != ' ' && line[j] != '\t' && line[j] != ',' && line[j] != '/') ++j;
            out.push_back(line.substr(i, j - i));
            i = j;
        }
        if (stop && (int)out.size() < n) return false;
    }
    return true;
}

bool ListReader::doubles(double *v, int n)
{
    std::vector<std::string> t;
    if (!tokens(t, n)) return false;
    for (int i = 0; i < n; ++i)
        if (!parse_double(t[i], v[i])) return false;
    return true;
}

bool ListReader::floats(float *v, int n)
{
    std::vector<std::string> t;
    if (!tokens(t, n)) return false;
    for (int i = 0; i < n; ++i)
        if (!parse_float(t[i], v[i])) return false;
    return true;
}

bool ListReader::ints(int *v, int n)
{
    std::vector<std::string> t;
    if (!tokens(t, n)) return false;
    for (int i = 0; i < n; ++i)
        if (!parse_int(t[i], v[i])) return false;
    return true;
}

bool read_in_file(const std::string &path, InFile &in, std::string &err)
{
    ListReader r(path);
    if (!r.ok()) { err = "cannot open " + path; return false; }
    std::string line;
    auto text = [&](std::string &dst) {
        if (!r.record(line)) return false;
        dst = a20(line);
        return true;
    };
    auto skip = [&]() { return r.record(line); };
    double two[2];
    const bool good = skip() && skip() && skip() && text(in.sources) && text(in.itimes) &&
                      text(in.receivers) && text(in.gridv) && r.doubles(&in.earth, 1) && r.ints(&in.fom, 1) &&
                      r.ints(&in.ltfr, 1) && r.doubles(two, 2) && skip() && skip() && skip() &&
                      r.ints(&in.fsrt, 1) && text(in.rtravel) && r.ints(&in.cfd, 1) && text(in.frechet);
    if (!good) { err = path + ": unreadable near line " + std::to_string(r.line_number() + 1); return false; }
    in.cslat = two[0];
    in.cslong = two[1];
    return true;
}

bool read_vtx(const std::string &path, Vtx &v, std::string &err)
{
    ListReader r(path);
    if (!r.ok()) { err = "cannot open " + path; return false; }
    int n3[3];
    double d3[3];
    bool good = r.ints(n3, 3);
    if (good) { v.nvr = n3[0]; v.nvx = n3[1]; v.nvz = n3[2]; }
    good = good && r.doubles(d3, 3);
    if (good) { v.gor = d3[0]; v.goxd = d3[1]; v.gozd = d3[2]; }
    good = good && r.doubles(d3, 3);
    if (good) { v.dvr = d3[0]; v.dvxd = d3[1]; v.dvzd = d3[2]; }
    good = good && r.ints(n3, 3);
    if (good) { v.nnr = n3[0]; v.nnx = n3[1]; v.nnz = n3[2]; }
    good = good && r.doubles(d3, 3);
    if (good) { v.rgor = d3[0]; v.rgoxd = d3[1]; v.rgozd = d3[2]; }
    good = good && r.doubles(d3, 3);
    if (good) { v.dnr = d3[0]; v.dnxd = d3[1]; v.dnzd = d3[2]; }
    if (!good) { err = path + ": bad grid header near line " + std::to_string(r.line_number() + 1); return false; }
    if (v.nvr < 1 || v.nvx < 1 || v.nvz < 1 || v.nnr < 2 || v.nnx < 2 || v.nnz < 2) {
        err = path + ": bad grid dimensions";
        return false;
    }
    const size_t n = (size_t)(v.nvr + 2) * (v.nvx + 2) * (v.nvz + 2);
    v.velv.resize(n);
    // F:6118-6125: DO i=0,nvz+1; DO j=0,nvx+1; DO k=0,nvr+1; READ(10,*) velv(k,j,i)
    for (size_t q = 0; q < n; ++q)
        if (!r.doubles(&v.velv[q], 1)) {
            err = path + ": expected " + std::to_string(n) + " velocity values, read " + std::to_string(q);
            return false;
        }
    return true;
}

bool read_sources(const std::string &path, SourceFile &s, std::string &err)
{
    ListReader r(path);
    if (!r.ok()) { err = "cannot open " + path; return false; }
    int nra = 0;
    if (!r.ints(&nra, 1) || nra < 0) { err = path + ": bad array count"; return false; }
    s.arrays.assign(nra, {});
    std::string line;
    for (int a = 0; a < nra; ++a) {
        int nsrc = 0;
        if (!r.ints(&nsrc, 1) || nsrc < 0) { err = path + ": bad source count of array " + std::to_string(a + 1); return false; }
        for (int i = 0; i < nsrc; ++i) {
            double v[3];
            if (!r.doubles(v, 3) || !r.record(line)) {   // lat lon depth, then the (a8) phase record
                err = path + ": bad source " + std::to_string(i + 1) + " of array " + std::to_string(a + 1);
                return false;
            }
            s.arrays[a].push_back({v[0], v[1], v[2], trim(line.substr(0, line.size() < 8 ? line.size() : 8))});
        }
    }
    return true;
}

bool read_receivers(const std::string &path, ReceiverFile &rf, std::string &err)
{
    ListReader r(path);
    if (!r.ok()) { err = "cannot open " + path; return false; }
    int nra = 0;
    if (!r.ints(&nra, 1) || nra < 0) { err = path + ": bad array count"; return false; }
    rf.arrays.assign(nra, {});
    for (int a = 0; a < nra; ++a) {
        int nrc = 0;
        if (!r.ints(&nrc, 1) || nrc < 0) { err = path + ": bad receiver count of array " + std::to_string(a + 1); return false; }
        for (int i = 0; i < nrc; ++i) {
            double v[3];
            if (!r.doubles(v, 3)) {
                err = path + ": bad receiver " + std::to_string(i + 1) + " of array " + std::to_string(a + 1);
                return false;
            }
            rf.arrays[a].push_back({v[0], v[1], v[2]});
        }
    }
    return true;
}

FrameReader::FrameReader(const std::string &path, int nnx, int nnz)
{
    f_ = std::fopen(path.c_str(), "rb");
    frame_ = (size_t)nnx * nnz;
}

FrameReader::~FrameReader()
{
    if (f_) std::fclose(f_);
}

bool FrameReader::next(int n, double *out)
{
    if (!f_) return false;
    const size_t want = frame_ * (size_t)n;
    return std::fread(out, sizeof(double), want, f_) == want;
}

std::string format_real4(float v)
{
    // gfortran writes a REAL(4) list item as 1X then G16.9E2 (9 significant
    // digits): F editing with 9-(exponent+1) decimals in 12 columns plus 4
    // blanks for 0.1 <= |v| < 1e9, E editing otherwise.
    char buf[64];
    std::string body;
    const double x = (double)v;
    if (x == 0.0) {
        body = std::signbit(x) ? "-0.00000000    " : "0.00000000    ";
        std::snprintf(buf, sizeof buf, "%16s", body.c_str());
        return " " + std::string(buf);
    }
    if (!std::isfinite(x)) {
        std::snprintf(buf, sizeof buf, "%16s", std::isnan(x) ? "NaN" : (x > 0 ? "Infinity" : "-Infinity"));
        return " " + std::string(buf);
    }
    char e[48];
    std::snprintf(e, sizeof e, "%.8E", x);     // rounded mantissa and its exponent
    const char *ep = std::strchr(e, 'E');
    const int e10 = std::atoi(ep + 1);
    if (e10 >= -1 && e10 <= 8) {
        char f[48];
        std::snprintf(f, sizeof f, "%.*f", 8 - e10, x);
        std::snprintf(buf, sizeof buf, "%12s    ", f);
    } else {
        std::string m(e, ep - e);
        char ex[16];
        if (std::abs(e10) < 100)
            std::snprintf(ex, sizeof ex, "E%c%02d", e10 < 0 ? '-' : '+', std::abs(e10));
        else
            std::snprintf(ex, sizeof ex, "%c%03d", e10 < 0 ? '-' : '+', std::abs(e10));
        std::snprintf(buf, sizeof buf, "%16s", (m + ex).c_str());
    }
    return " " + std::string(buf);
}

bool read_frechet(const std::string &path, int64_t nrows, std::vector<int64_t> &row_ptr, std::vector<int32_t> &cols,
                  std::vector<float> &vals, std::string &err)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) { err = "cannot open " + path; return false; }
    auto rec = [&](int32_t &a, float &b) {
        int32_t l0 = 0, l1 = 0;
        if (std::fread(&l0, 4, 1, f) != 1 || l0 != 8 || std::fread(&a, 4, 1, f) != 1 || std::fread(&b, 4, 1, f) != 1 ||
            std::fread(&l1, 4, 1, f) != 1 || l1 != 8)
            return false;
        return true;
    };
    if (row_ptr.empty()) row_ptr.push_back((int64_t)cols.size());
    bool good = true;
    for (int64_t r = 0; r < nrows && good; ++r) {
        int32_t n = 0;
        float recid = 0.0f;
        if (!rec(n, recid) || n < 0) { good = false; break; }
        for (int32_t k = 0; k < n; ++k) {
            int32_t c = 0;
            float v = 0.0f;
            if (!rec(c, v)) { good = false; break; }
            cols.push_back(c);
            vals.push_back(v);
        }
        row_ptr.push_back((int64_t)cols.size());
    }
    std::fclose(f);
    if (!good) err = path + ": truncated or malformed record";
    return good;
}

std::string format_real8(double v)
{
    char buf[64];
    std::snprintf(buf, sizeof buf, " %24.17E", v);
    return buf;
}

FrechetWriter::FrechetWriter(const std::string &path) { f_ = std::fopen(path.c_str(), "wb"); }

FrechetWriter::~FrechetWriter()
{
    if (f_) std::fclose(f_);
}

bool FrechetWriter::rec(int32_t a, float b)
{
    const int32_t len = 8;
    return std::fwrite(&len, 4, 1, f_) == 1 && std::fwrite(&a, 4, 1, f_) == 1 && std::fwrite(&b, 4, 1, f_) == 1 &&
           std::fwrite(&len, 4, 1, f_) == 1;
}

bool FrechetWriter::row(int receiver, const int32_t *cols, const float *vals, int64_t n)
{
    if (!f_ || !rec((int32_t)n, (float)receiver)) return false;
    for (int64_t i = 0; i < n; ++i)
        if (!rec(cols[i], vals[i])) return false;
    return true;
}

bool FrechetWriter::empty_row() { return f_ && rec(0, 0.0f); }

}  // namespace fm3dt_io
