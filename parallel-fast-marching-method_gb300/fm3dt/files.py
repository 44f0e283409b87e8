"""Readers and writers of the reference program's files.

Formats (fm3dt_parallel.f90 = "F", subinv.f90 = "S"):

* ``fm3dt_parallel.in`` -- 18 positional lines (F:6082-6102); file names are
  read (a20), numbers list-directed, trailing text ignored.
* velocity grid ``.vtx`` -- six header lines (F:6103-6108), then one velocity
  per record, r fastest, over the (nvr+2)(nvx+2)(nvz+2) padded nodes
  (F:6118-6125); only the first value of each record is read.
* ``sources.dat`` -- nra; per array nsrc, then per source a "lat lon depth"
  record and a phase record (F:6275-6282).
* ``receivers.dat`` -- nra; per array nrc, then "elev_km lat lon [name]"
  per receiver (F:6286-6315).
* ``itimes.out`` -- raw native doubles, nnz*nnx per source (phi fastest),
  sources back to back (F:6215-6219, 6907).
* ``rtravel.out`` -- one list-directed REAL(4) per record, source-major,
  receiver-minor (F:7174-7176).
* ``frechet.out`` -- gfortran unformatted sequential records of (int32,
  float32); per row a header (entries, real(receiver index)) and then one
  (1-based column, value) record per entry (F:6589-6595, read by S:351-391).
* ``otimes.dat`` -- per source-receiver pair "tstat residual uncertainty"
  (read by S:349).
"""
from __future__ import annotations

import struct
from dataclasses import dataclass, field

import numpy as np


def _list_values(lines, n, pos, conv=float):
    """List-directed read of n values starting at record ``pos``; returns
    (values, next record index).  Blank records are skipped; the rest of the
    last record used is discarded."""
    out = []
    while len(out) < n:
        if pos >= len(lines):
            raise ValueError("unexpected end of file")
        toks = lines[pos].replace(",", " ").split()
        pos += 1
        for t in toks:
            if t.startswith("/"):
                break
            out.append(t)
            if len(out) == n:
                break
    return [conv(t.replace("d", "e").replace("D", "e")) for t in out], pos


def _a20(line: str) -> str:
    return line[:20].strip()


@dataclass
class InFile:
    sources: str = "sources.dat"
    itimes: str = "itimes.out"
    receivers: str = "receivers.dat"
    gridv: str = "gridc.vtx"
    earth: float = 6371.0
    fom: int = 1
    ltfr: int = 1
    cslat: float = 0.4
    cslong: float = 0.4
    fsrt: int = 1
    rtravel: str = "rtravel.out"
    cfd: int = 1
    frechet: str = "frechet.out"


def write_in_file(path, f: InFile):
    c = "c" * 70

    def row(v, text):
        return f"{str(v):<23}c: {text}\n"

    with open(path, "w") as fh:
        fh.write(c + "\nc INPUT PARAMETERS\n" + c + "\n")
        fh.write(row(f.sources, "File containing source information"))
        fh.write(row(f.itimes, "File containing initial traveltimes"))
        fh.write(row(f.receivers, "File containing receiver positions"))
        fh.write(row(f.gridv, "File containing velocity grid information"))
        fh.write(row(repr(float(f.earth)), "Earth radius in km"))
        fh.write(row(f.fom, "Use first-order(0) or mixed-order(1) scheme"))
        fh.write(row(f.ltfr, "Limit traveltime field to receivers (0=no,1=yes)"))
        fh.write(row(f"{f.cslat}     {f.cslong}", "(lat,lon) cushion around receiver array (degrees)"))
        fh.write(c + "\nc OUTPUT FILES\n" + c + "\n")
        fh.write(row(f.fsrt, "find source-receiver traveltimes (0=no,1=yes)"))
        fh.write(row(f.rtravel, "Name of file containing source-receiver traveltimes"))
        fh.write(row(f.cfd, "Calculate partial (Frechet) derivatives (0=no,1=yes)"))
        fh.write(row(f.frechet, "Name of file containing Frechet derivatives"))


def read_in_file(path) -> InFile:
    lines = open(path).read().splitlines()
    f = InFile()
    f.sources, f.itimes, f.receivers, f.gridv = (_a20(lines[i]) for i in range(3, 7))
    pos = 7
    (f.earth,), pos = _list_values(lines, 1, pos)
    (f.fom,), pos = _list_values(lines, 1, pos, int)
    (f.ltfr,), pos = _list_values(lines, 1, pos, int)
    (f.cslat, f.cslong), pos = _list_values(lines, 2, pos)
    pos += 3
    (f.fsrt,), pos = _list_values(lines, 1, pos, int)
    f.rtravel = _a20(lines[pos])
    pos += 1
    (f.cfd,), pos = _list_values(lines, 1, pos, int)
    f.frechet = _a20(lines[pos])
    return f


@dataclass
class GridHeader:
    """The six .vtx header lines (degrees and km, as in the file)."""
    nv: tuple
    vorig: tuple
    vstep: tuple
    nn: tuple
    norig: tuple
    nstep: tuple
    earth: float = 6371.0


def write_vtx(path, h, velv, second_column: float | None = 0.0, fmt: str = "%.17g"):
    """Writes a .vtx grid file.  ``velv`` is r fastest over the padded node
    grid; each record holds the velocity and, if given, a second column
    that the solver does not read."""
    velv = np.asarray(velv, dtype=np.float64).ravel()
    nvr, nvx, nvz = h.nv
    if velv.size != (nvr + 2) * (nvx + 2) * (nvz + 2):
        raise ValueError("velv has %d values, grid needs %d" % (velv.size, (nvr + 2) * (nvx + 2) * (nvz + 2)))
    with open(path, "w") as fh:
        # header values keep every digit (shortest exact decimal form)
        real3 = (lambda v: "".join(" %11s" % repr(float(x)) for x in v) + "\n")
        fh.write("%12d%12d%12d\n" % tuple(h.nv))
        fh.write(real3(h.vorig))
        fh.write(real3(h.vstep))
        fh.write("%12d%12d%12d\n" % tuple(h.nn))
        fh.write(real3(h.norig))
        fh.write(real3(h.nstep))
        fh.write("\n")
        tail = "" if second_column is None else "  " + (fmt % second_column)
        fh.write("".join("  " + (fmt % v) + tail + "\n" for v in velv))


def read_vtx(path, earth: float = 6371.0):
    """(GridHeader, velv) of a .vtx file; header values exactly as written."""
    lines = open(path).read().splitlines()
    nv, pos = _list_values(lines, 3, 0, int)
    vo, pos = _list_values(lines, 3, pos)
    vs, pos = _list_values(lines, 3, pos)
    nn, pos = _list_values(lines, 3, pos, int)
    no, pos = _list_values(lines, 3, pos)
    ns, pos = _list_values(lines, 3, pos)
    n = (nv[0] + 2) * (nv[1] + 2) * (nv[2] + 2)
    vals = []
    for line in lines[pos:]:
        t = line.replace(",", " ").split()
        if t:
            vals.append(float(t[0].replace("d", "e").replace("D", "e")))
            if len(vals) == n:
                break
    if len(vals) != n:
        raise ValueError(f"{path}: expected {n} velocity values, found {len(vals)}")
    h = GridHeader(tuple(nv), tuple(vo), tuple(vs), tuple(nn), tuple(no), tuple(ns), earth)
    return h, np.array(vals)


def write_sources(path, arrays):
    """arrays: list (per receiver array) of lists of (lat, lon, depth, phase)."""
    with open(path, "w") as fh:
        fh.write(f"{len(arrays)}\n")
        for arr in arrays:
            fh.write(f"{len(arr):12d}\n")
            for lat, lon, dep, ph in arr:
                fh.write(f"  {lat:.6f}       {lon:.4f}       {dep:.5f}    \n  {ph:<7s}\n")


def read_sources(path):
    lines = open(path).read().splitlines()
    (nra,), pos = _list_values(lines, 1, 0, int)
    arrays = []
    for _ in range(nra):
        (ns,), pos = _list_values(lines, 1, pos, int)
        arr = []
        for _ in range(ns):
            (lat, lon, dep), pos = _list_values(lines, 3, pos)
            arr.append((lat, lon, dep, lines[pos][:8].strip()))
            pos += 1
        arrays.append(arr)
    return arrays


def write_receivers(path, arrays):
    """arrays: list of lists of (elev_km, lat, lon, name)."""
    with open(path, "w") as fh:
        fh.write(f"{len(arrays)}\n")
        for a, arr in enumerate(arrays):
            fh.write(f"{len(arr)}         ARRAY {a + 1}\n")
            for el, lat, lon, name in arr:
                fh.write(f"{float(el)!r}     {float(lat)!r}    {float(lon)!r}     {name}\n")


def read_receivers(path):
    lines = open(path).read().splitlines()
    (nra,), pos = _list_values(lines, 1, 0, int)
    arrays = []
    for _ in range(nra):
        (nr,), pos = _list_values(lines, 1, pos, int)
        arr = []
        for _ in range(nr):
            v, pos = _list_values(lines, 3, pos)
            arr.append(tuple(v))
        arrays.append(arr)
    return arrays


def write_itimes(path, frames):
    np.ascontiguousarray(frames, dtype="=f8").tofile(path)


def read_itimes(path, nnx, nnz):
    d = np.fromfile(path, dtype="=f8")
    return d.reshape(-1, nnx * nnz)


def read_rtravel(path) -> np.ndarray:
    return np.array([float(t) for t in open(path).read().split()], dtype=np.float32)


def format_real4(v) -> str:
    """gfortran's list-directed record for one REAL(4) value (1X, G16.9E2),
    e.g. 357.198395 -> '   357.198395    '."""
    x = float(np.float32(v))
    if x == 0.0:
        return " " + "%16s" % "0.00000000    "
    m, e = ("%.8E" % x).split("E")
    e10 = int(e)
    if -1 <= e10 <= 8:
        return " " + "%12s    " % ("%.*f" % (8 - e10, x))
    ex = "E%s%02d" % ("-" if e10 < 0 else "+", abs(e10)) if abs(e10) < 100 else "%s%03d" % (
        "-" if e10 < 0 else "+", abs(e10))
    return " " + "%16s" % (m + ex)


def write_rtravel(path, times):
    with open(path, "w") as fh:
        fh.write("".join(format_real4(t) + "\n" for t in np.asarray(times, dtype=np.float32).ravel()))


@dataclass
class FrechetRows:
    """Rows of frechet.out: per row its receiver index (the header's real
    value) and its (1-based column, value) entries in file order."""
    row_ptr: np.ndarray
    cols: np.ndarray
    vals: np.ndarray
    recid: np.ndarray = field(default=None)


def write_frechet(path, row_ptr, cols, vals, recid):
    row_ptr = np.asarray(row_ptr, dtype=np.int64)
    cols = np.asarray(cols, dtype=np.int32)
    vals = np.asarray(vals, dtype=np.float32)
    rec = struct.Struct("=iifi")
    with open(path, "wb") as fh:
        for q in range(len(row_ptr) - 1):
            a, b = row_ptr[q], row_ptr[q + 1]
            fh.write(rec.pack(8, int(b - a), float(recid[q]), 8))
            for j in range(a, b):
                fh.write(rec.pack(8, int(cols[j]), float(vals[j]), 8))


def read_frechet(path) -> FrechetRows:
    raw = np.fromfile(path, dtype=np.uint8)
    if raw.size % 16:
        raise ValueError(f"{path}: {raw.size} bytes is not a whole number of 16-byte records")
    rec = raw.view(np.dtype([("l0", "=i4"), ("a", "=i4"), ("b", "=f4"), ("l1", "=i4")]))
    if rec.size and (np.any(rec["l0"] != 8) or np.any(rec["l1"] != 8)):
        raise ValueError(f"{path}: record markers are not 8")
    ptr, recid, cols, vals = [0], [], [], []
    i = 0
    while i < rec.size:
        n = int(rec["a"][i])
        recid.append(float(rec["b"][i]))
        cols.append(rec["a"][i + 1:i + 1 + n])
        vals.append(rec["b"][i + 1:i + 1 + n])
        if len(cols[-1]) != n:
            raise ValueError(f"{path}: truncated row {len(recid)}")
        ptr.append(ptr[-1] + n)
        i += 1 + n
    cat = (lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt))
    return FrechetRows(np.array(ptr, np.int64), cat(cols, np.int32), cat(vals, np.float32),
                       np.array(recid, np.float64))


SUBINV_KEYS = [("gridi", "a"), ("gridc", "a"), ("otimes", "a"), ("rtimes", "a"), ("mtimes", "a"),
               ("rmtr", "i"), ("frechet", "a"), ("sources", "a"), ("receivers", "a"), ("subiter", "a"),
               ("epsilon", "f"), ("subdim", "i"), ("asds", "i"), ("eta", "f"), ("invst", "i"),
               ("stfile", "a"), ("stdf", "f"), ("fracg", "f"), ("earth", "f")]


def write_subinv_in(path, **kw):
    """subinv.in: three comment records, then one item per
    record; file names are read (a25)."""
    defaults = dict(gridi="gridi.vtx", gridc="gridc.vtx", otimes="otimes.dat", rtimes="rtimes.dat",
                    mtimes="rtravel.out", rmtr=1, frechet="frechet.out", sources="sources.dat",
                    receivers="receivers.dat", subiter="subiter.in", epsilon=10.0, subdim=10, asds=1, eta=10.0,
                    invst=0, stfile="stationres.dat", stdf=10.0, fracg=0.1, earth=6371.0)
    defaults.update(kw)
    c = "c" * 70
    with open(path, "w") as fh:
        fh.write(c + "\nc INPUT PARAMETERS\n" + c + "\n")
        for k, _ in SUBINV_KEYS:
            fh.write(f"{str(defaults[k]):<26}c: {k}\n")


def read_subinv_in(path) -> dict:
    lines = open(path).read().splitlines()
    out, pos = {}, 3
    for k, t in SUBINV_KEYS:
        if t == "a":
            out[k] = lines[pos][:25].strip()
            pos += 1
        else:
            (v,), pos = _list_values(lines, 1, pos, int if t == "i" else float)
            out[k] = v
    return out


def write_otimes(path, tstat, resid, unc):
    with open(path, "w") as fh:
        for s, r, u in zip(tstat, resid, unc):
            fh.write("%12d %12.7f %16.7E\n" % (int(s), float(r), float(u)))


def read_otimes(path):
    t, r, u = [], [], []
    for line in open(path):
        f = line.split()
        if len(f) >= 3:
            t.append(int(f[0]))
            r.append(float(f[1].replace("d", "e").replace("D", "e")))
            u.append(float(f[2].replace("d", "e").replace("D", "e")))
    return np.array(t, np.int32), np.array(r), np.array(u)
