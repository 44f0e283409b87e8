"""The oracle's restatement of the reference's decomposed run (no GPU).

The reference's production layout is mpirun -np 9: eight compute ranks in a
2 x 2 x 2 block split plus a file writer (fm3dt_parallel.f90 F:6052-6056).
Each rank marches its own block with local_fmm, and bulk-synchronous rounds
exchange two ghost layers per face, re-solve the boundary nodes a ghost can
lower with the face stencils (order_overlap, F:157-416; fouds2_left ..
fouds2_down, F:1100-2825) and stop when no node moved by more than 1e-5 s
(F:6371-6451).  oracle.fmm_decomposed emulates those ranks.  Pinned here:
* one block is the serial run, bit for bit (same gridder, seed and march);
* the face stencils' branch bodies are fouds2_all's (checked against the
  reference source in this container when it is present);
* the decomposed run is a different discretisation near block faces: it
  differs from the serial march by amounts that shrink with the spacing on a
  one-axis split, and the 2 x 2 x 2 run stops within a few rounds with every
  node set;
* the rounds give the same field with the blocks of a round run in turn or
  on threads.
"""
import os
import re

import numpy as np
import pytest

REF = "/root/reference/fm3dt_parallel.f90"


def _case(orc, cfg, scale, ev=None):
    from fm3dt import synth
    w = synth.config(cfg, scale=scale, nev=1)
    if ev is not None:
        w.events = np.array([ev], dtype=np.float64)
    h = w.header
    g = orc.grid_from_header(h.nv, h.vorig, h.vstep, h.nn, h.norig, h.nstep, h.earth)
    veln, _ = orc.gridder(g, w.velv)
    frame = orc.planewave_frame(g, orc.PlaneWave(*synth.planewave_params(h, *w.events[0])))
    return w, g, veln, frame


@pytest.mark.parametrize("cfg,scale", [(0, 20), (1, 22), (2, 18)])
def test_one_block_is_the_serial_march(orc, cfg, scale):
    w, g, veln, frame = _case(orc, cfg, scale)
    serial, _ = orc.fmm(g, veln, frame, 1)
    dec, rounds = orc.fmm_decomposed(g, w.velv, frame, 1, (1, 1, 1))
    assert np.array_equal(dec, serial)
    assert rounds == 1


def test_one_axis_split_converges_to_the_serial_march(orc):
    """Next to a block face the blocks' own stencils lose their second-order
    term (the second neighbour lies in the other block), so the decomposed
    field differs from the serial one there; the difference falls with the
    spacing."""
    diffs = []
    for n in (16, 32, 64):
        w, g, veln, frame = _case(orc, 0, n)
        serial, _ = orc.fmm(g, veln, frame, 1)
        dec, rounds = orc.fmm_decomposed(g, w.velv, frame, 1, (2, 1, 1))
        assert rounds <= 4
        assert np.all(dec > 0)
        diffs.append(float(np.max(np.abs(dec - serial))))
    assert diffs[1] < diffs[0] and diffs[2] < diffs[1]
    assert diffs[2] < 0.02


def test_eight_blocks_stop_and_fill_the_grid(orc):
    w, g, veln, frame = _case(orc, 0, 32)
    serial, _ = orc.fmm(g, veln, frame, 1)
    dec, rounds = orc.fmm_decomposed(g, w.velv, frame, 1, (2, 2, 2))
    assert 2 <= rounds <= 8
    assert np.all(dec > 0)
    # the bottom frame is fixed in both runs
    n = g.nnz * g.nnx
    assert np.array_equal(dec[-n:], serial[-n:])
    # the block holding the earliest boundary time is marched exactly as the
    # serial run marches it (nothing reaches it from the others)
    d = (dec - serial).reshape(g.nnr, g.nnx, g.nnz)
    fr = frame.reshape(g.nnx, g.nnz)
    ix, iz = np.unravel_index(np.argmin(np.where(fr > 0, fr, np.inf)), fr.shape)
    sx = slice(0, g.nnx // 2) if ix < g.nnx // 2 else slice(g.nnx // 2, g.nnx)
    sz = slice(0, g.nnz // 2) if iz < g.nnz // 2 else slice(g.nnz // 2, g.nnz)
    assert np.max(np.abs(d[g.nnr // 2:, sx, sz])) < 1e-9


def test_threads_do_not_change_the_rounds(orc, monkeypatch):
    w, g, veln, frame = _case(orc, 1, 24)
    a, ra = orc.fmm_decomposed(g, w.velv, frame, 1, (2, 2, 2))
    monkeypatch.setenv("ORC_DECOMPOSED_THREADS", "1")
    b, rb = orc.fmm_decomposed(g, w.velv, frame, 1, (2, 2, 2))
    assert ra == rb
    assert np.array_equal(a, b)


def _bodies(lines):
    out, cur = [], []
    for l in lines:
        t = l.strip()
        if t.startswith(("IF(", "ELSEIF(", "ELSE IF(", "ENDIF")) or t == "ELSE":
            if cur:
                out.append(tuple(cur))
                cur = []
            continue
        if "=" in t and not t.startswith("sw"):
            cur.append(re.sub(r"\s+", "", t))
    if cur:
        out.append(tuple(cur))
    return out


def _table(src, name):
    s = src.index(f"SUBROUTINE {name}(")
    e = src.index(f"END SUBROUTINE {name}", s)
    block = src[s:e].split("\n")
    i0 = next(i for i, l in enumerate(block) if "swsol=0" in l)
    i1 = next(i for i, l in enumerate(block) if "IF(swsol.EQ.1)" in l)
    return block[i0:i1]


@pytest.mark.skipif(not os.path.exists(REF), reason="reference source not present")
def test_face_stencils_are_fouds2_all_with_the_ghost_axis_used():
    """The restatement evaluates each face stencil with fouds2_all's branch
    table (the ghost neighbour always taken); the reference's six face
    routines hold exactly those branch bodies, in that order, once the ghost
    values are written as the neighbour they stand for."""
    src = open(REF).read()
    allb = _bodies(_table(src, "fouds2_all"))
    subs = {
        "left": [("ttn_ghost_left(iz,2,ir)", "ttn(iz,j,ir)"), ("ttn_ghost_left(iz,1,ir)", "ttn(iz,j2,ir)")],
        "right": [("ttn_ghost_right(iz,1,ir)", "ttn(iz,j,ir)"), ("ttn_ghost_right(iz,2,ir)", "ttn(iz,j2,ir)")],
        "in": [("ttn_ghost_in(2,ix,ir)", "ttn(k,ix,ir)"), ("ttn_ghost_in(1,ix,ir)", "ttn(k2,ix,ir)")],
        "out": [("ttn_ghost_out(1,ix,ir)", "ttn(k,ix,ir)"), ("ttn_ghost_out(2,ix,ir)", "ttn(k2,ix,ir)")],
        "up": [("ttn_ghost_up(iz,ix,2)", "ttn(iz,ix,i)"), ("ttn_ghost_up(iz,ix,1)", "ttn(iz,ix,i2)")],
        "down": [("ttn_ghost_down(iz,ix,1)", "ttn(iz,ix,i)"), ("ttn_ghost_down(iz,ix,2)", "ttn(iz,ix,i2)")],
    }
    axis = {"left": "ttn(iz,j,ir)", "right": "ttn(iz,j,ir)", "in": "ttn(k,ix,ir)", "out": "ttn(k,ix,ir)",
            "up": "ttn(iz,ix,i)", "down": "ttn(iz,ix,i)"}
    for face, sb in subs.items():
        txt = "\n".join(_table(src, f"fouds2_{face}"))
        for a, b in sb:
            txt = txt.replace(a, b)
        fb = _bodies(txt.split("\n"))
        with_ghost = [b for b in allb if any(axis[face] in st for st in b)]
        assert fb == with_ghost, face
