"""Seeded synthetic workloads for the forward traveltime solve.

The reference's own end-to-end input (the itimes.out boundary-time file) is
not available, and no public benchmark exists for this path, so every
workload here is synthetic and seeded with ``numpy.random.default_rng``:

* geometry: a spherical section 0-400 km deep and 10 x 10 degrees wide,
  centred at 35 S 145 E, earth radius 6371 km (the reference's
  fm3dt_parallel.in value);
* velocity: a linear 5.8 -> 8.9 km/s gradient with depth on a cubic B-spline
  node grid, plus a per-workload perturbation (checkerboard, Gaussian node
  noise or a dipping slow slab);
* boundary times: a teleseismic plane wave on the bottom face, described per
  event by its epicentral distance and back-azimuth (the distance law is a
  smooth synthetic relation stated in ``planewave_params``; no global
  reference-earth table is used);
* receivers: uniform random surface positions inside the section.

Header values follow the .vtx convention of the reference (heights in km,
latitude/longitude in degrees; fm3dt_parallel.f90:6103-6108).
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np


@dataclass
class Header:
    """The six header lines of a .vtx velocity file (fm3dt_parallel.f90:6103-6108)."""
    nv: tuple          # nvr, nvx, nvz (interior velocity nodes)
    vorig: tuple       # gor (km height), goxd (latitude, deg), gozd (longitude, deg)
    vstep: tuple       # dvr (km), dvxd (deg), dvzd (deg)
    nn: tuple          # nnr, nnx, nnz (propagation nodes)
    norig: tuple       # rgor, rgoxd, rgozd
    nstep: tuple       # dnr, dnxd, dnzd
    earth: float = 6371.0


def section_header(nnr, nnx, nnz, nvr, nvx, nvz, depth_km=400.0, width_deg=10.0,
                   lat_c=-35.0, lon_c=145.0, earth=6371.0) -> Header:
    """Propagation grid spanning the section exactly, with a velocity node
    grid whose B-spline support covers every propagation node including the
    reference's ghost layer (indices -1..n+1), so no velocity index is ever
    clamped."""
    dnr = depth_km / (nnr - 1)
    dnxd = width_deg / (nnx - 1)
    dnzd = width_deg / (nnz - 1)
    rgor = 0.0
    rgoxd = lat_c + 0.5 * width_deg       # northern edge: x runs southwards
    rgozd = lon_c - 0.5 * width_deg
    m = 2.05                                # velocity origin 2.05 fine cells outside
    gor = rgor + m * dnr
    goxd = rgoxd + m * dnxd
    gozd = rgozd - m * dnzd
    dvr = (nnr + m) * dnr / (nvr - 1.5)
    dvxd = (nnx + m) * dnxd / (nvx - 1.5)
    dvzd = (nnz + m) * dnzd / (nvz - 1.5)
    return Header((nvr, nvx, nvz), (gor, goxd, gozd), (dvr, dvxd, dvzd),
                  (nnr, nnx, nnz), (rgor, rgoxd, rgozd), (dnr, dnxd, dnzd), earth)


def _node_depths(h: Header):
    nvr = h.nv[0]
    heights = h.vorig[0] - (np.arange(nvr + 2) - 1.0) * h.vstep[0]
    return -heights


def velocity_model(h: Header, kind: str, seed: int) -> np.ndarray:
    """velv values in .vtx order: (nvz+2, nvx+2, nvr+2) with r fastest,
    flattened.  kind: 'checker', 'gauss', 'slab' or 'plain'."""
    nvr, nvx, nvz = h.nv
    depth = _node_depths(h)                                  # (nvr+2,)
    base = 5.8 + (8.9 - 5.8) * depth / 400.0
    v = np.broadcast_to(base[None, None, :], (nvz + 2, nvx + 2, nvr + 2)).copy()
    rng = np.random.default_rng(seed)
    iz, ix, ir = np.meshgrid(np.arange(nvz + 2), np.arange(nvx + 2), np.arange(nvr + 2), indexing="ij")
    if kind == "checker":
        sign = np.where(((iz // 3) + (ix // 3) + (ir // 3)) % 2 == 0, 1.0, -1.0)
        v *= 1.0 + 0.05 * sign
    elif kind == "gauss":
        pert = np.clip(rng.normal(0.0, 0.015, v.shape), -0.03, 0.03)
        v *= 1.0 + pert
    elif kind == "slab":
        # slow slab dipping 45 degrees: distance of a node from the plane
        # depth = (x - x0) through the section centre, 15% contrast, 60 km thick
        km_per_deg = math.pi / 180.0 * h.earth
        xkm = (ix - 1.0) * h.vstep[1] * km_per_deg
        x0 = 0.5 * (nvx - 1) * h.vstep[1] * km_per_deg
        d = np.abs((depth[ir] - (xkm - x0) - 100.0) / math.sqrt(2.0))
        slab = np.where(d < 30.0, -0.15, 0.0)
        noise = rng.normal(0.0, 0.10 / 3.0, v.shape)
        v *= (1.0 + slab) * (1.0 + np.clip(noise, -0.10, 0.10))
    elif kind != "plain":
        raise ValueError(kind)
    return np.ascontiguousarray(v.reshape(-1))


def receivers(h: Header, n: int, seed: int):
    """Surface receivers (elevation 0 km) at uniform random lat/lon strictly
    inside the section, one propagation cell away from its lateral faces."""
    rng = np.random.default_rng(seed)
    nnr, nnx, nnz = h.nn
    lat_n = h.norig[1] - h.nstep[1]
    lat_s = h.norig[1] - (nnx - 2) * h.nstep[1]
    lon_w = h.norig[2] + h.nstep[2]
    lon_e = h.norig[2] + (nnz - 2) * h.nstep[2]
    lat = rng.uniform(lat_s, lat_n, n)
    lon = rng.uniform(lon_w, lon_e, n)
    elev = np.zeros(n)
    return elev, lat, lon


def planewave_params(h: Header, delta_deg: float, baz_deg: float):
    """Synthetic teleseismic plane wave of one event (boundary-time
    injection): arrival time t0 under the section centre at the bottom face,
    horizontal slowness p along the bottom surface (s/km), and the
    propagation azimuth.  The distance law t0 = 150 + 10*D - 0.025*D^2 s
    (D in degrees) is synthetic; its derivative gives p."""
    d2r = math.pi / 180.0
    rb = h.earth + (h.norig[0] - (h.nn[0] - 1) * h.nstep[0])
    t0 = 150.0 + 10.0 * delta_deg - 0.025 * delta_deg * delta_deg
    p = (10.0 - 0.05 * delta_deg) / (rb * d2r)
    az = (baz_deg + 180.0) * d2r
    return (t0, p, math.cos(az), math.sin(az))


@dataclass
class Workload:
    name: str
    header: Header
    velv: np.ndarray
    events: np.ndarray            # (nev, 2): delta_deg, baz_deg
    rec_elev: np.ndarray
    rec_lat: np.ndarray
    rec_lon: np.ndarray
    seen: np.ndarray = field(default=None)   # (nev, nrc) bool picks mask


def config(idx: int, nev: int | None = None, scale: int | None = None) -> Workload:
    """The five synthetic workloads.  ``scale`` overrides the propagation grid
    edge (for small parity cases with the same structure); ``nev`` the event
    count."""
    seed = idx * 1000 + 1
    rng = np.random.default_rng(seed)
    if idx == 0:
        n = scale or 64
        h = section_header(n, n, n, 12, 14, 14)
        kind, nrc, ne = "checker", 100, nev or 1
    elif idx == 1:
        n = scale or 128
        h = section_header(n, n, n, 12, 14, 14)
        kind, nrc, ne = "gauss", 300, nev or 256
    elif idx == 2:
        n = scale or 256
        h = section_header(n, n, n, 16, 20, 20)
        kind, nrc, ne = "slab", 300, nev or 16
    elif idx == 3:
        if scale:
            nr, nx, nz = scale, scale * 7 // 6, scale * 7 // 6
        else:
            nr, nx, nz = 192, 224, 224
        h = section_header(nr, nx, nz, 16, 20, 20)
        kind, nrc, ne = "checker", 300, nev or 500
    else:
        raise ValueError(idx)
    velv = velocity_model(h, kind, seed)
    if idx == 0 and ne == 1:
        events = np.array([[60.0, 45.0]])
    else:
        events = np.stack([rng.uniform(30.0, 90.0, ne), rng.uniform(0.0, 360.0, ne)], axis=1)
    elev, lat, lon = receivers(h, nrc, seed + 7)
    seen = None
    if idx == 1:
        frac = rng.uniform(0.7, 1.0, nrc)
        seen = rng.uniform(0.0, 1.0, (ne, nrc)) < frac[None, :]
    return Workload(f"config{idx}", h, velv, events, elev, lat, lon, seen)


def planewave_frames(h: Header, params) -> np.ndarray:
    """Boundary frames (nev, nnx*nnz, phi fastest) of the synthetic plane
    waves, with the formula of the device generator: t = t0 + p * d, d the
    tangent-plane distance of a bottom node from the section centre along the
    propagation azimuth.  Angles converted like fm3dt_parallel.f90:6110-6117."""
    pi = float(np.float32(3.1415926535898))
    nnr, nnx, nnz = h.nn
    dnr = h.nstep[0]
    dnx = h.nstep[1] * pi / 180.0
    dnz = h.nstep[2] * pi / 180.0
    rgox = (90.0 - h.norig[1]) * pi / 180.0
    rgoz = h.norig[2] * pi / 180.0
    rb = h.earth + (h.norig[0] - (nnr - 1) * dnr)
    thc = rgox + (nnx - 1) * dnx * 0.5
    phc = rgoz + (nnz - 1) * dnz * 0.5
    rbs = rb * math.sin(thc)
    th = rgox + np.arange(nnx, dtype=np.float64) * dnx
    ph = rgoz + np.arange(nnz, dtype=np.float64) * dnz
    dn = rb * (thc - th)                  # (nnx,)
    de = rbs * (ph - phc)                 # (nnz,)
    params = np.asarray(params, dtype=np.float64).reshape(-1, 4)
    out = np.empty((len(params), nnx, nnz))
    for e, (t0, p, ca, sa) in enumerate(params):
        out[e] = t0 + p * (dn[:, None] * ca + de[None, :] * sa)
    return out.reshape(len(params), nnx * nnz)


@dataclass
class TomographyProblem:
    """A teleseismic tomography run: the starting model (a 1-D gradient, as
    gridi.vtx holds it: 8 decimals, a priori standard deviation 0.3), the
    true model (the config-3 checkerboard), and a survey of plane-wave
    sources and surface receivers, array by array."""
    header: Header
    velv_start: np.ndarray
    velv_true: np.ndarray
    cm_sd: np.ndarray
    frames: list                  # per array (nsrc, nnx*nnz)
    receivers: list               # per array (nrc, 3): elev km, lat, lon
    events: list                  # per array (nsrc, 2): distance, back-azimuth


def tomography_problem(scale: int | None = None, arrays=((500, 300),), seed: int = 3001) -> TomographyProblem:
    w = config(3, nev=1, scale=scale)
    h = w.header
    # as the solver reads gridi.vtx written with 8 decimals
    start = np.array([float("%.8f" % v) for v in velocity_model(h, "plain", seed)])
    true = velocity_model(h, "checker", seed)
    rng = np.random.default_rng(seed)
    frames, recs, evs = [], [], []
    for a, (ns, nr) in enumerate(arrays):
        ev = np.stack([rng.uniform(30.0, 90.0, ns), rng.uniform(0.0, 360.0, ns)], axis=1)
        params = np.array([planewave_params(h, *e) for e in ev])
        frames.append(planewave_frames(h, params))
        elev, lat, lon = receivers(h, nr, seed + 11 + a)
        recs.append(np.stack([elev, lat, lon], axis=1))
        evs.append(ev)
    return TomographyProblem(h, start, true, np.full(start.size, 0.3, np.float32), frames, recs, evs)
