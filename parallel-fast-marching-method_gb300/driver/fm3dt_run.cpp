// fm3dt_run -- the reference program's file contract on one GB300.
//
// Replaces `mpirun -np 9 ./fm3dt_parallel` (run in a working directory with
// no arguments, sub.sh:23): reads fm3dt_parallel.in and the files it names,
// solves every source of every array through libfm3dt_gpu, and writes
// rtravel.out (fsrt = 1) and frechet.out (cfd = 1) in the reference's order:
// array by array, source by source, receiver by receiver (F:6273-6599).
//
//   fm3dt_run [-C dir] [--in file] [--precision fp64|fp32] [--batch N] [--check]
//   fm3dt_run --print-real4 value...
//
// --check parses every input and prints a JSON summary without touching the
// GPU; --print-real4 prints each value as one rtravel.out record.  Exit
// status: 0 success, 1 unreadable or inconsistent input, 2 a library error
// (its message on stderr).
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>
#include <vector>

#include <unistd.h>

#include "../../include/fm3dt_gpu.h"
#include "fm3dt_files.h"

using namespace fm3dt_io;

namespace {

struct Args {
    std::string dir, in = "fm3dt_parallel.in";
    int precision = FM3DT_FP64;
    int batch = 512;
    bool check = false;
};

int usage()
{
    std::fprintf(stderr, "usage: fm3dt_run [-C dir] [--in file] [--precision fp64|fp32] [--batch N] [--check]\n");
    return 1;
}

// fm3dt_parallel.f90:61 sets its double-precision pi from a single-precision
// literal; receivers convert with that value (F:6313-6314).
double ref_pi() { return (double)3.1415926535898f; }

int input_error(const std::string &msg)
{
    std::fprintf(stderr, "fm3dt_run: %s\n", msg.c_str());
    return 1;
}

int lib_error(fm3dt_ctx *ctx, const char *what, int rc)
{
    std::fprintf(stderr, "fm3dt_run: %s failed (%d): %s\n", what, rc, fm3dt_last_error(ctx));
    return 2;
}

long file_size(const std::string &path)
{
    FILE *f = std::fopen(path.c_str(), "rb");
    if (!f) return -1;
    std::fseek(f, 0, SEEK_END);
    const long n = std::ftell(f);
    std::fclose(f);
    return n;
}

}  // namespace

int main(int argc, char **argv)
{
    Args a;
    if (argc > 1 && std::strcmp(argv[1], "--print-real4") == 0) {
        // one rtravel.out record per argument (format check)
        for (int i = 2; i < argc; ++i) std::printf("%s\n", format_real4(std::strtof(argv[i], nullptr)).c_str());
        return 0;
    }
    for (int i = 1; i < argc; ++i) {
        const std::string s = argv[i];
        if (s == "-C" && i + 1 < argc) a.dir = argv[++i];
        else if (s == "--in" && i + 1 < argc) a.in = argv[++i];
        else if (s == "--precision" && i + 1 < argc) {
            const std::string p = argv[++i];
            if (p == "fp64") a.precision = FM3DT_FP64;
            else if (p == "fp32") a.precision = FM3DT_FP32_OFFSET;
            else return usage();
        } else if (s == "--batch" && i + 1 < argc) {
            a.batch = std::atoi(argv[++i]);
            if (a.batch < 1) return usage();
        } else if (s == "--check") a.check = true;
        else return usage();
    }
    if (!a.dir.empty() && chdir(a.dir.c_str()) != 0) return input_error("cannot enter " + a.dir);

    std::string err;
    InFile in;
    if (!read_in_file(a.in, in, err)) return input_error(err);
    Vtx v;
    if (!read_vtx(in.gridv, v, err)) return input_error(err);
    SourceFile src;
    if (!read_sources(in.sources, src, err)) return input_error(err);
    ReceiverFile rec;
    const bool need_rec = in.fsrt == 1 || in.cfd == 1 || in.ltfr == 1;
    if (need_rec) {
        if (!read_receivers(in.receivers, rec, err)) return input_error(err);
        if (rec.arrays.size() != src.arrays.size()) {
            // the reference's message and stop (F:6179-6189)
            std::fprintf(stderr, "ERROR!!!\nSource and receiver files are\ninconsistent!!!!\n"
                                 "First line of each file should\nbe identical!!!\nTERMINATING PROGRAM!!!\n");
            return 1;
        }
    }
    size_t total_src = 0;
    for (auto &arr : src.arrays) total_src += arr.size();
    const size_t frame = (size_t)v.nnx * v.nnz;
    const long isz = file_size(in.itimes);
    if (isz < 0) return input_error("cannot open " + in.itimes);
    if ((size_t)isz < total_src * frame * sizeof(double))
        return input_error(in.itimes + ": " + std::to_string(isz) + " bytes, " + std::to_string(total_src) +
                           " sources need " + std::to_string(total_src * frame * sizeof(double)));

    if (a.check) {
        double vsum = 0.0;
        for (double x : v.velv) vsum += x;
        FrameReader fr(in.itimes, v.nnx, v.nnz);
        std::vector<double> buf(frame);
        double tsum = 0.0;
        for (size_t i = 0; i < total_src; ++i) {
            if (!fr.next(1, buf.data())) return input_error(in.itimes + ": short read");
            for (double x : buf) tsum += x;
        }
        std::printf("{\"sources\": \"%s\", \"itimes\": \"%s\", \"receivers\": \"%s\", \"gridv\": \"%s\", "
                    "\"earth\": %.17g, \"fom\": %d, \"ltfr\": %d, \"cslat\": %.17g, \"cslong\": %.17g, "
                    "\"fsrt\": %d, \"rtravel\": \"%s\", \"cfd\": %d, \"frechet\": \"%s\", ",
                    in.sources.c_str(), in.itimes.c_str(), in.receivers.c_str(), in.gridv.c_str(), in.earth,
                    in.fom, in.ltfr, in.cslat, in.cslong, in.fsrt, in.rtravel.c_str(), in.cfd, in.frechet.c_str());
        std::printf("\"nv\": [%d, %d, %d], \"vorig\": [%.17g, %.17g, %.17g], \"vstep\": [%.17g, %.17g, %.17g], "
                    "\"nn\": [%d, %d, %d], \"norig\": [%.17g, %.17g, %.17g], \"nstep\": [%.17g, %.17g, %.17g], "
                    "\"velv_n\": %zu, \"velv_sum\": %.17g, ",
                    v.nvr, v.nvx, v.nvz, v.gor, v.goxd, v.gozd, v.dvr, v.dvxd, v.dvzd, v.nnr, v.nnx, v.nnz,
                    v.rgor, v.rgoxd, v.rgozd, v.dnr, v.dnxd, v.dnzd, v.velv.size(), vsum);
        std::printf("\"nsrc\": [");
        for (size_t i = 0; i < src.arrays.size(); ++i) std::printf("%s%zu", i ? ", " : "", src.arrays[i].size());
        std::printf("], \"nrc\": [");
        for (size_t i = 0; i < rec.arrays.size(); ++i) std::printf("%s%zu", i ? ", " : "", rec.arrays[i].size());
        std::printf("], \"first_phase\": \"%s\", \"itimes_sum\": %.17g}\n",
                    total_src ? src.arrays[0][0].phase.c_str() : "", tsum);
        return 0;
    }

    fm3dt_grid_desc d{};
    d.nvr = v.nvr; d.nvx = v.nvx; d.nvz = v.nvz;
    d.gor = v.gor; d.goxd = v.goxd; d.gozd = v.gozd;
    d.dvr = v.dvr; d.dvxd = v.dvxd; d.dvzd = v.dvzd;
    d.nnr = v.nnr; d.nnx = v.nnx; d.nnz = v.nnz;
    d.rgor = v.rgor; d.rgoxd = v.rgoxd; d.rgozd = v.rgozd;
    d.dnr = v.dnr; d.dnxd = v.dnxd; d.dnzd = v.dnzd;
    d.earth = in.earth;
    d.fom = in.fom;
    d.precision = a.precision;
    size_t max_nsrc = 1;
    for (auto &arr : src.arrays) max_nsrc = arr.size() > max_nsrc ? arr.size() : max_nsrc;
    d.max_events = (int)(max_nsrc < (size_t)a.batch ? max_nsrc : (size_t)a.batch);

    fm3dt_ctx *ctx = nullptr;
    int rc = fm3dt_ctx_create(&d, &ctx);
    if (rc != FM3DT_OK) return lib_error(ctx, "fm3dt_ctx_create", rc);
    rc = fm3dt_set_velocity(ctx, v.velv.data());
    if (rc != FM3DT_OK) { const int e = lib_error(ctx, "fm3dt_set_velocity", rc); fm3dt_ctx_destroy(ctx); return e; }

    FILE *rt = nullptr;
    if (in.fsrt == 1) {
        rt = std::fopen(in.rtravel.c_str(), "w");
        if (!rt) { fm3dt_ctx_destroy(ctx); return input_error("cannot write " + in.rtravel); }
    }
    FrechetWriter *fw = nullptr;
    if (in.cfd == 1) {
        fw = new FrechetWriter(in.frechet);
        if (!fw->ok()) { fm3dt_ctx_destroy(ctx); return input_error("cannot write " + in.frechet); }
    }
    FrameReader frames(in.itimes, v.nnx, v.nnz);
    const double pi = ref_pi();
    std::vector<double> fbuf((size_t)d.max_events * frame);
    std::vector<float> times;
    std::vector<int64_t> row_ptr;
    std::vector<int32_t> cols;
    std::vector<float> vals;
    int status = 0;
    size_t done = 0;
    for (size_t ai = 0; ai < src.arrays.size() && !status; ++ai) {
        const size_t nsrc = src.arrays[ai].size();
        std::vector<double> rcr, rcx, rcz;
        if (need_rec)
            for (const Receiver &r : rec.arrays[ai]) {
                rcr.push_back(r.elev);
                rcx.push_back((90.0 - r.lat) * pi / 180.0);
                rcz.push_back(r.lon * pi / 180.0);
            }
        const int nrc = (int)rcr.size();
        for (size_t s0 = 0; s0 < nsrc && !status; s0 += (size_t)d.max_events) {
            const int nb = (int)((nsrc - s0) < (size_t)d.max_events ? (nsrc - s0) : (size_t)d.max_events);
            if (!frames.next(nb, fbuf.data())) { status = input_error(in.itimes + ": short read"); break; }
            fm3dt_status st{};
            const size_t rows = (size_t)nb * nrc;
            // With both outputs, one forward call (solve, times, rays and rows;
            // the rays of the batch's faster part start while the rest still
            // solves); a capacity too small for the rows solves once more.
            const bool forward = rt && fw && nrc > 0;
            if (forward) {
                times.resize(rows);
                row_ptr.assign(rows + 1, 0);
                int64_t cap = (int64_t)rows * 512;
                for (int attempt = 0; attempt < 2; ++attempt) {
                    cols.resize((size_t)cap);
                    vals.resize((size_t)cap);
                    rc = fm3dt_forward(ctx, nb, fbuf.data(), nrc, rcr.data(), rcx.data(), rcz.data(), times.data(),
                                       row_ptr.data(), cols.data(), vals.data(), cap, nullptr, &st);
                    if (rc == FM3DT_ERANGE && row_ptr[rows] > cap) { cap = row_ptr[rows]; continue; }
                    break;
                }
                if (rc != FM3DT_OK) { status = lib_error(ctx, "fm3dt_forward", rc); break; }
            } else {
                rc = fm3dt_solve(ctx, nb, fbuf.data(), &st);
                if (rc != FM3DT_OK) { status = lib_error(ctx, "fm3dt_solve", rc); break; }
            }
            for (int e = 0; e < nb; ++e)
                std::printf("Finish Source: %zu (array %zu) rounds %d\n", s0 + e + 1, ai + 1, st.rounds);
            if (rt && nrc > 0) {
                if (!forward) {
                    times.resize(rows);
                    rc = fm3dt_receiver_times(ctx, nrc, rcr.data(), rcx.data(), rcz.data(), times.data());
                    if (rc != FM3DT_OK) { status = lib_error(ctx, "fm3dt_receiver_times", rc); break; }
                }
                for (float t : times) std::fprintf(rt, "%s\n", format_real4(t).c_str());
            }
            if (fw && nrc > 0) {
                if (!forward) {
                    row_ptr.assign(rows + 1, 0);
                    int64_t cap = (int64_t)rows * 512;
                    for (int attempt = 0; attempt < 2; ++attempt) {
                        cols.resize((size_t)cap);
                        vals.resize((size_t)cap);
                        rc = fm3dt_rays_frechet(ctx, nrc, rcr.data(), rcx.data(), rcz.data(), row_ptr.data(),
                                                cols.data(), vals.data(), cap, nullptr);
                        if (rc == FM3DT_ERANGE && row_ptr[rows] > cap) { cap = row_ptr[rows]; continue; }
                        break;
                    }
                    if (rc != FM3DT_OK) { status = lib_error(ctx, "fm3dt_rays_frechet", rc); break; }
                }
                for (size_t q = 0; q < rows; ++q) {
                    const int k = (int)(q % nrc) + 1;   // receiver index within its array
                    if (!fw->row(k, cols.data() + row_ptr[q], vals.data() + row_ptr[q], row_ptr[q + 1] - row_ptr[q])) {
                        status = input_error("cannot write " + in.frechet);
                        break;
                    }
                }
            }
            done += nb;
        }
    }
    if (rt) std::fclose(rt);
    delete fw;
    fm3dt_ctx_destroy(ctx);
    if (!status) std::fprintf(stderr, "fm3dt_run: %zu sources solved\n", done);
    return status;
}
