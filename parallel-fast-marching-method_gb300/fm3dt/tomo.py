"""Teleseismic tomography driver: the reference's sub.sh loop on one GB300.

sub.sh (sub.sh:15-40) alternates the forward program and subinv through
files: forward solve of the starting model, its receiver times copied to
rtimes.dat as the reference times, then five times (subinv, forward solve).
Two drivers here:

* ``Tomography`` keeps everything in one process: the boundary frames of
  every source stay resident on the GPU across iterations, each iteration's
  receiver times and Frechet rows come back to the host for the subspace
  step (host code by design), and the new model goes back to the GPU.  The
  values passed between the stages go through the same REAL(4) text forms
  the files impose (rtravel.out, gridc.vtx), so the in-process loop and the
  file loop compute the same models.
* ``run_workdir`` runs the programs fm3dt_run and fm3dt_subinv in a
  reference-style working directory exactly as sub.sh runs fm3dt_parallel
  and subinv.
"""
from __future__ import annotations

import os
import shutil
import subprocess
from dataclasses import dataclass, field

import numpy as np

from . import files as F
from . import subinv as SI


def real4_text(x) -> np.ndarray:
    """The double a REAL(8) list-directed read gets from a REAL(4) value
    written list-directed (gridc.vtx written by subinv, read by the forward
    solver): the 9-significant-digit decimal of the float."""
    x = np.asarray(x, dtype=np.float32).ravel()
    return np.array([float(F.format_real4(v)) for v in x])


@dataclass
class Survey:
    """Sources and receivers, array by array (sources.dat / receivers.dat)
    with each source's boundary frame (its itimes.out record)."""
    frames: list                     # per array: (nsrc, nnx*nnz) float64
    receivers: list                  # per array: (nrc, 3) elev km, lat deg, lon deg

    @property
    def nsrc(self):
        return np.array([len(f) for f in self.frames], dtype=np.int32)

    @property
    def nrc(self):
        return np.array([len(r) for r in self.receivers], dtype=np.int32)


@dataclass
class Iteration:
    model: np.ndarray                # velocity the forward solve used (float64, .vtx order)
    times: np.ndarray                # receiver times (float32, rtravel.out order)
    subdim: int = 0
    rms_residual: float = 0.0        # picked (model - reference - observed) residuals, seconds
    note: str = ""
    dm: np.ndarray = None            # the subspace step that produced this model


@dataclass
class History:
    iterations: list = field(default_factory=list)


class Tomography:
    """In-process sub.sh.  ``header``: grids; ``velv_ref``: the starting
    model as the forward solver reads it (gridi.vtx velocities, float64);
    ``cm_sd``: gridi.vtx's second column; ``survey``: sources and receivers;
    ``params``: subinv.in values; ``schedule``: the solver's solve schedule
    (tie_sweeps, tie_ratio, resweeps, resweep_frac; see
    ``Solver.set_schedule``), None for the library's defaults."""

    def __init__(self, header, velv_ref, cm_sd, survey: Survey, params: SI.Params, precision=None,
                 subinv_precision=SI.FP32, batch: int = 512, fom: int = 1, schedule=None):
        import fm3dt
        import torch
        self.header = header
        self.velv_ref = np.asarray(velv_ref, dtype=np.float64)
        self.mo = self.velv_ref.astype(np.float32)
        self.cm_sd = np.asarray(cm_sd, dtype=np.float32)
        self.survey = survey
        self.params = params
        self.subinv_precision = subinv_precision
        prec = fm3dt.FP32_OFFSET if precision is None else precision
        nmax = max(int(np.max(survey.nsrc)), 1)
        self.batch = min(batch, nmax)
        self.solver = fm3dt.Solver(header, fom=fom, precision=prec, max_events=self.batch)
        if schedule is not None:
            self.solver.set_schedule(*schedule)
        # boundary frames resident in device memory for every iteration
        self.d_frames = [torch.from_numpy(np.ascontiguousarray(f, dtype=np.float64)).cuda() for f in survey.frames]
        self.rec = []
        for r in survey.receivers:
            r = np.asarray(r, dtype=np.float64).reshape(-1, 3)
            rcx, rcz = fm3dt.latlon_to_rad(r[:, 1], r[:, 2])
            self.rec.append((np.ascontiguousarray(r[:, 0]), rcx, rcz))
        self.grid = (tuple(header.nv), tuple(header.vorig), tuple(header.vstep))

    def close(self):
        self.solver.close()

    def forward(self, velv):
        """Receiver times (float32, source-major per array) and Frechet rows
        (CSR, one row per source-receiver pair) of one model."""
        self.solver.set_velocity(velv)
        times, ptrs, cols, vals = [], [np.zeros(1, np.int64)], [], []
        base = 0
        for a, d_fr in enumerate(self.d_frames):
            rcr, rcx, rcz = self.rec[a]
            n = d_fr.shape[0]
            for s0 in range(0, n, self.batch):
                nb = min(self.batch, n - s0)
                self.solver.solve_ptr(nb, d_fr[s0:s0 + nb].data_ptr(), True)
                times.append(self.solver.receiver_times(rcr, rcx, rcz).ravel())
                rp, c, v, _ = self.solver.rays_frechet(rcr, rcx, rcz)
                ptrs.append(rp[1:] + base)
                base += int(rp[-1])
                cols.append(c)
                vals.append(v)
        cat = (lambda xs, dt: np.concatenate(xs).astype(dt) if xs else np.zeros(0, dt))
        return (cat(times, np.float32), np.concatenate(ptrs), cat(cols, np.int32), cat(vals, np.float32))

    def run(self, iterations: int, tstat, dobs, cd_sd) -> History:
        """sub.sh: reference solve, then ``iterations`` x (subinv, solve)."""
        h = History()
        model = self.velv_ref.copy()
        times, rp, cols, vals = self.forward(model)
        rtimes = times.copy()                   # cp rtravel.out rtimes.dat
        h.iterations.append(Iteration(model, times, rms_residual=self._rms(times, rtimes, tstat, dobs)))
        nmpv = self.mo.size
        nmps = int(np.sum(self.survey.nrc)) if self.params.invst == 1 else 0
        mc = np.concatenate([self.mo, np.zeros(nmps, np.float32)])   # subiter 1: mc = mo, station terms 0
        for _ in range(iterations):
            dm, used, note = SI.step(self.grid, self.params, self.survey.nsrc, self.survey.nrc, self.mo,
                                     self.cm_sd, mc, tstat, dobs, cd_sd, times, rtimes, rp, cols, vals,
                                     self.subinv_precision)
            if self.subinv_precision == SI.FP32:
                new = (mc + dm.astype(np.float32)).astype(np.float32)
            else:
                new = (mc.astype(np.float64) + dm).astype(np.float32)
            model = real4_text(new[:nmpv])             # gridc.vtx as the solver reads it
            # and as subinv reads gridc.vtx and the station-term file back
            mc = np.concatenate([model.astype(np.float32), new[nmpv:]])
            times, rp, cols, vals = self.forward(model)
            h.iterations.append(Iteration(model, times, used, self._rms(times, rtimes, tstat, dobs), note, dm))
        return h

    @staticmethod
    def _rms(times, rtimes, tstat, dobs):
        m = np.asarray(tstat) == 1
        if not np.any(m):
            return 0.0
        r = (times.astype(np.float64) - rtimes)[m] - np.asarray(dobs, dtype=np.float64)[m]
        return float(np.sqrt(np.mean(r * r)))


def run_workdir(workdir: str, iterations: int = 5, forward_args=(), subinv_args=()):
    """sub.sh in ``workdir`` (which holds fm3dt_parallel.in, subinv.in and
    their files, with gridi.vtx the starting model and gridc.vtx the
    forward solver's model file).  Returns the exit codes."""
    from . import build as fb
    fb.build_driver()
    fb.build_subinv()
    sub = F.read_subinv_in(os.path.join(workdir, "subinv.in"))
    fin = F.read_in_file(os.path.join(workdir, "fm3dt_parallel.in"))

    def run(cmd):
        r = subprocess.run(cmd, cwd=workdir, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f"{os.path.basename(cmd[0])} failed ({r.returncode}):\n{r.stdout}\n{r.stderr}")
        return r

    shutil.copyfile(os.path.join(workdir, sub["gridi"]), os.path.join(workdir, sub["gridc"]))
    with open(os.path.join(workdir, sub["subiter"]), "w") as fh:
        fh.write("1\n")
    run([fb.DRIVER, *forward_args])
    shutil.copyfile(os.path.join(workdir, fin.rtravel), os.path.join(workdir, sub["rtimes"]))
    for it in range(1, iterations + 1):
        run([fb.SUBINV, *subinv_args])
        run([fb.DRIVER, *forward_args])
        with open(os.path.join(workdir, sub["subiter"]), "w") as fh:
            fh.write(f"{it + 1}\n")
