// fm3dt_subinv -- one subspace inversion step with the reference's files.
//
// Replaces `./subinv` (sub.sh:29): reads subinv.in and the files
// it names, runs fm3dt_subinv_step, and writes the new model to the current
// grid file and, with station terms, the station-term file
// (S:513-519).
//
//   fm3dt_subinv [-C dir] [--in subinv.in] [--precision fp32|fp64]
//
// Exit status: 0 success, 1 unreadable or inconsistent input, 2 an error of
// the inversion (its message on stderr).
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <unistd.h>

#include "../../include/fm3dt_subinv.h"
#include "../driver/fm3dt_files.h"

using namespace fm3dt_io;

namespace {

// (a25) file names
std::string a25(const std::string &line)
{
    std::string s = line.substr(0, line.size() < 25 ? line.size() : 25);
    size_t a = 0, b = s.size();
    while (a < b && (s[a] == ' ' || s[a] == '\t')) ++a;
    while (b > a && (s[b - 1] == ' ' || s[b - 1] == '\t' || s[b - 1] == '\r')) --b;
    return s.substr(a, b - a);
}

int input_error(const std::string &m)
{
    std::fprintf(stderr, "fm3dt_subinv: %s\n", m.c_str());
    return 1;
}

struct Params {
    std::string gridi, gridc, otimes, rtimes, mtimes, frechet, sources, receive, subiter, stfile;
    fm3dt_subinv_desc d{};
};

bool read_params(const std::string &path, Params &p, std::string &err)
{
    ListReader r(path);
    if (!r.ok()) { err = "cannot open " + path; return false; }
    std::string line;
    auto name = [&](std::string &dst) {
        if (!r.record(line)) return false;
        dst = a25(line);
        return true;
    };
    const bool good = r.record(line) && r.record(line) && r.record(line) && name(p.gridi) && name(p.gridc) &&
                      name(p.otimes) && name(p.rtimes) && name(p.mtimes) && r.ints(&p.d.rmtr, 1) &&
                      name(p.frechet) && name(p.sources) && name(p.receive) && name(p.subiter) &&
                      r.floats(&p.d.epsilon, 1) && r.ints(&p.d.subdim, 1) && r.ints(&p.d.asds, 1) &&
                      r.floats(&p.d.eta, 1) && r.ints(&p.d.invst, 1) && name(p.stfile) && r.floats(&p.d.stdf, 1) &&
                      r.floats(&p.d.fracg, 1) && r.floats(&p.d.earth, 1);
    if (!good) err = path + ": unreadable near line " + std::to_string(r.line_number() + 1);
    return good;
}

// nra and the per-array source and receiver counts
bool read_counts(const Params &p, std::vector<int> &nsrc, std::vector<int> &nrc, std::string &err)
{
    SourceFile s;
    ReceiverFile r;
    if (!read_sources(p.sources, s, err) || !read_receivers(p.receive, r, err)) return false;
    if (s.arrays.size() != r.arrays.size()) {
        err = "ERROR!!!\nSource and receiver files are\ninconsistent!!!!\nFirst line of each file should\n"
              "be identical!!!\nTERMINATING PROGRAM!!!";
        return false;
    }
    for (size_t a = 0; a < s.arrays.size(); ++a) {
        nsrc.push_back((int)s.arrays[a].size());
        nrc.push_back((int)r.arrays[a].size());
    }
    return true;
}

}  // namespace

int main(int argc, char **argv)
{
    std::string dir, in = "subinv.in";
    int precision = FM3DT_SUBINV_FP32;
    for (int i = 1; i < argc; ++i) {
        const std::string s = argv[i];
        if (s == "-C" && i + 1 < argc) dir = argv[++i];
        else if (s == "--in" && i + 1 < argc) in = argv[++i];
        else if (s == "--precision" && i + 1 < argc) {
            const std::string v = argv[++i];
            if (v == "fp32") precision = FM3DT_SUBINV_FP32;
            else if (v == "fp64") precision = FM3DT_SUBINV_FP64;
            else return input_error("bad precision " + v);
        } else {
            std::fprintf(stderr, "usage: fm3dt_subinv [-C dir] [--in subinv.in] [--precision fp32|fp64]\n");
            return 1;
        }
    }
    if (!dir.empty() && chdir(dir.c_str()) != 0) return input_error("cannot enter " + dir);
    std::string err;
    Params p;
    if (!read_params(in, p, err)) return input_error(err);
    p.d.precision = precision;
    int invstep = 0;
    {
        ListReader r(p.subiter);
        if (!r.ok() || !r.ints(&invstep, 1)) return input_error("cannot read " + p.subiter);
    }
    std::vector<int> nsrc, nrc;
    if (!read_counts(p, nsrc, nrc, err)) return input_error(err);
    int ntr = 0, nmps = 0;
    for (size_t a = 0; a < nsrc.size(); ++a) {
        ntr += nsrc[a] * nrc[a];
        nmps += nrc[a];
    }
    // reference grid: header, then (velocity, a priori sd) per node
    ListReader gi(p.gridi);
    if (!gi.ok()) return input_error("cannot open " + p.gridi);
    int n3[3], a3[3];
    double g3[3], d3[3], b3[3], c3[3];
    if (!gi.ints(n3, 3) || !gi.doubles(g3, 3) || !gi.doubles(d3, 3) || !gi.ints(a3, 3) || !gi.doubles(b3, 3) ||
        !gi.doubles(c3, 3))
        return input_error(p.gridi + ": bad header");
    p.d.nvr = n3[0]; p.d.nvt = n3[1]; p.d.nvp = n3[2];
    p.d.gor = g3[0]; p.d.got = g3[1]; p.d.gop = g3[2];
    p.d.dnr = d3[0]; p.d.dnt = d3[1]; p.d.dnp = d3[2];
    const int nmpv = (n3[0] + 2) * (n3[1] + 2) * (n3[2] + 2);
    const int nmp = nmpv + (p.d.invst == 1 ? nmps : 0);
    std::vector<float> mo(nmpv), cm(nmpv), mc(nmp, 0.0f);
    for (int i = 0; i < nmpv; ++i) {
        float v[2];
        if (!gi.floats(v, 2)) return input_error(p.gridi + ": expected " + std::to_string(nmpv) + " node records");
        mo[i] = v[0];
        cm[i] = v[1];
        mc[i] = v[0];
    }
    if (invstep > 1) {
        ListReader gc(p.gridc);
        std::string line;
        for (int i = 0; i < 6; ++i)
            if (!gc.record(line)) return input_error(p.gridc + ": bad header");
        for (int i = 0; i < nmpv; ++i)
            if (!gc.floats(&mc[i], 1)) return input_error(p.gridc + ": short");
    }
    if (p.d.invst == 1 && invstep > 1) {
        ListReader st(p.stfile);
        for (int i = nmpv; i < nmp; ++i)
            if (!st.floats(&mc[i], 1)) return input_error(p.stfile + ": short");
    }
    // residuals, model and reference times, Frechet rows
    std::vector<int> tstat(ntr);
    std::vector<float> dobs(ntr), cd(ntr), mt(ntr), rt(ntr);
    {
        // list-directed "tstat dobs cd" records
        FILE *f = std::fopen(p.otimes.c_str(), "r");
        if (!f) return input_error("cannot open " + p.otimes);
        for (int i = 0; i < ntr; ++i)
            if (std::fscanf(f, "%d %f %f%*[^\n]", &tstat[i], &dobs[i], &cd[i]) != 3) {
                std::fclose(f);
                return input_error(p.otimes + ": bad record " + std::to_string(i + 1));
            }
        std::fclose(f);
    }
    {
        ListReader mm(p.mtimes), rr(p.rtimes);
        for (int i = 0; i < ntr; ++i)
            if (!mm.floats(&mt[i], 1) || !rr.floats(&rt[i], 1))
                return input_error(p.mtimes + " / " + p.rtimes + ": short at record " + std::to_string(i + 1));
    }
    std::vector<int64_t> row_ptr;
    std::vector<int32_t> cols;
    std::vector<float> vals;
    if (!read_frechet(p.frechet, ntr, row_ptr, cols, vals, err)) return input_error(err);
    std::vector<double> dm(nmp);
    int used = 0;
    char msg[1024];
    const int rc = fm3dt_subinv_step(&p.d, (int)nsrc.size(), nsrc.data(), nrc.data(), mo.data(), cm.data(), mc.data(),
                                     tstat.data(), dobs.data(), cd.data(), mt.data(), rt.data(), row_ptr.data(),
                                     cols.data(), vals.data(), dm.data(), &used, msg, (int)sizeof msg);
    if (msg[0]) std::printf("%s", msg);
    if (rc != FM3DT_SUBINV_OK) {
        std::fprintf(stderr, "fm3dt_subinv: inversion failed (%d)\n", rc);
        return 2;
    }
    // new model: the header as read, then mc + dm in REAL(4)
    FILE *out = std::fopen(p.gridc.c_str(), "w");
    if (!out) return input_error("cannot write " + p.gridc);
    std::fprintf(out, "%12d%12d%12d\n", n3[0], n3[1], n3[2]);
    std::fprintf(out, "%s%s%s\n", format_real8(g3[0]).c_str(), format_real8(g3[1]).c_str(), format_real8(g3[2]).c_str());
    std::fprintf(out, "%s%s%s\n", format_real8(d3[0]).c_str(), format_real8(d3[1]).c_str(), format_real8(d3[2]).c_str());
    std::fprintf(out, "%12d%12d%12d\n", a3[0], a3[1], a3[2]);
    std::fprintf(out, "%s%s%s\n", format_real8(b3[0]).c_str(), format_real8(b3[1]).c_str(), format_real8(b3[2]).c_str());
    std::fprintf(out, "%s%s%s\n", format_real8(c3[0]).c_str(), format_real8(c3[1]).c_str(), format_real8(c3[2]).c_str());
    const bool f32 = precision == FM3DT_SUBINV_FP32;
    for (int i = 0; i < nmpv; ++i) {
        const float v = f32 ? mc[i] + (float)dm[i] : (float)((double)mc[i] + dm[i]);
        std::fprintf(out, "%s\n", format_real4(v).c_str());
    }
    std::fclose(out);
    if (p.d.invst == 1) {
        FILE *st = std::fopen(p.stfile.c_str(), "w");
        if (!st) return input_error("cannot write " + p.stfile);
        for (int i = nmpv; i < nmp; ++i) {
            const float v = f32 ? mc[i] + (float)dm[i] : (float)((double)mc[i] + dm[i]);
            std::fprintf(st, "%s\n", format_real4(v).c_str());
        }
        std::fclose(st);
    }
    std::printf("subspace dimension %d, %d picked residuals, %d model parameters\n", used,
                (int)std::count(tstat.begin(), tstat.end(), 1), nmp);
    return 0;
}
