// fm3dt_files.h -- the reference program's input and output files.
//
// Readers follow the Fortran READ statements of fm3dt_parallel.f90 ("F"):
// list-directed reads take the first values of a record and skip the rest of
// it (so trailing "c: comment" text is ignored), continue over blank records,
// and accept Fortran 'd' exponents; (a20) reads take the first 20 characters.
// Writers produce what gfortran writes for the reference's WRITE statements.
#pragma once

#include <cstdint>
#include <cstdio>
#include <string>
#include <vector>

namespace fm3dt_io {

// fm3dt_parallel.in (F:6082-6102): 18 positional lines.
struct InFile {
    std::string sources, itimes, receivers, gridv;   // (a20) file names
    double earth = 0.0;
    int fom = 1;
    int ltfr = 0;                  // read and ignored, as in the reference (F:84-86)
    double cslat = 0.0, cslong = 0.0;
    int fsrt = 1;                  // write source-receiver times
    std::string rtravel;
    int cfd = 0;                   // write Frechet derivatives
    std::string frechet;
};

// Velocity grid file (.vtx, F:6103-6126): six header lines, then one value
// per record for r fastest, then theta, then phi, over the padded node grid.
struct Vtx {
    int nvr = 0, nvx = 0, nvz = 0;
    double gor = 0, goxd = 0, gozd = 0, dvr = 0, dvxd = 0, dvzd = 0;
    int nnr = 0, nnx = 0, nnz = 0;
    double rgor = 0, rgoxd = 0, rgozd = 0, dnr = 0, dnxd = 0, dnzd = 0;
    std::vector<double> velv;      // (nvr+2)(nvx+2)(nvz+2), r fastest
};

// One array of sources (F:6275-6282) or receivers (F:6286-6315); the
// coordinates are kept in the file's units (degrees, km).
struct Source { double lat, lon, depth; std::string phase; };
struct Receiver { double elev, lat, lon; };
struct SourceFile { std::vector<std::vector<Source>> arrays; };
struct ReceiverFile { std::vector<std::vector<Receiver>> arrays; };

// Record-oriented list-directed reader.
class ListReader {
public:
    explicit ListReader(const std::string &path);
    bool ok() const { return f_ != nullptr; }
    ~ListReader();
    // Reads n values starting at the next record, skipping blank records,
    // and discards the rest of the last record used.  False at end of file
    // or on a value that does not parse.
    bool doubles(double *out, int n);
    bool ints(int *out, int n);
    // REAL(4) items: each value converted from its decimal text to float
    bool floats(float *out, int n);
    // Reads one whole record (without its newline).
    bool record(std::string &line);
    long line_number() const { return line_no_; }

private:
    FILE *f_ = nullptr;
    long line_no_ = 0;
    bool tokens(std::vector<std::string> &out, int n);
};

bool read_in_file(const std::string &path, InFile &in, std::string &err);
bool read_vtx(const std::string &path, Vtx &v, std::string &err);
bool read_sources(const std::string &path, SourceFile &s, std::string &err);
bool read_receivers(const std::string &path, ReceiverFile &r, std::string &err);

// itimes.out: raw native doubles, nnz*nnx per source (phi fastest), sources
// back to back in file order across all arrays (F:6215-6219, 6907).
class FrameReader {
public:
    FrameReader(const std::string &path, int nnx, int nnz);
    ~FrameReader();
    bool ok() const { return f_ != nullptr; }
    // Reads the next n frames; false if the file ends first.
    bool next(int n, double *out);

private:
    FILE *f_ = nullptr;
    size_t frame_ = 0;
};

// Reads nrows rows of frechet.out (format below): per row its entries
// (1-based column, value) appended to cols/vals and row_ptr extended.
bool read_frechet(const std::string &path, int64_t nrows, std::vector<int64_t> &row_ptr, std::vector<int32_t> &cols,
                  std::vector<float> &vals, std::string &err);

// gfortran list-directed output of one REAL(8) value (17 significant digits).
std::string format_real8(double v);

// gfortran list-directed output of one REAL(4) value, one per record
// (WRITE(10,*) trr at F:7174-7176), e.g. "   357.198395    ".
std::string format_real4(float v);

// frechet.out, gfortran unformatted sequential (F:6589-6595): every record
// is a 4-byte length, an int32 and a float32, the length again.  Each row
// starts with a header record (entries, real(receiver index)) and is
// followed by one (1-based column, value) record per entry.
class FrechetWriter {
public:
    explicit FrechetWriter(const std::string &path);
    ~FrechetWriter();
    bool ok() const { return f_ != nullptr; }
    bool row(int receiver, const int32_t *cols, const float *vals, int64_t n);
    bool empty_row();

private:
    FILE *f_ = nullptr;
    bool rec(int32_t a, float b);
};

}  // namespace fm3dt_io
