"""FDPS-style walks and the MultiWalk loop, on the functor-compatible batch entry points.

A host that keeps FDPS and moves only the functors to the GPU hands the library
walks: an i-group of particles with its j-list, in the reference's payload
layouts (class.h EPI / EPJ / RESULT), through the dispatch / retrieve callbacks
of calcForceAllAndWriteBackMultiWalk (sph_dispatch_* / sph_retrieve_*).  This
module builds such walks for a whole particle state and drives them the way the
MultiWalk loop does, so the boundary can be measured on a full step:

* i-groups: the gravity groups of the device's octree (cells of at most n_group
  particles whose parent holds more, main.cpp:86-90), which partition the
  particles;
* gravity j-lists: the device's EPJ / SPJ lists of those groups at the opening
  angle (FDPS Monopole walk semantics, sph_get_grav_lists);
* SPH j-lists: FDPS Gather / Symmetry supersets -- every particle within
  2.5 h_max of the group's box (gather), and every particle within
  max(2.5 h_max, 2.5 h_j) of it (symmetric); as in FDPS, out-of-support j add
  zero to the sums and only enter the hydro functor's v_sig;
* the loop: walks in batches of n_walk_limit, batch b dispatched on tag
  b mod n_tags after the batch that last used that tag has been retrieved;
* two forms: the payload form (calcForceAllAndWriteBackMultiWalk: every walk
  carries copies of its j payloads) and the index form
  (calcForceAllAndWriteBackMultiWalkIndex: the pass's EPJ / SPJ arrays are
  sent once, with send_flag, and every walk carries int32 indices into them).

Used by bench.py's drop-in measurement; host-side numpy and scipy only.
"""
from __future__ import annotations

import ctypes as C
import time

import numpy as np

from . import layouts as T
from .ic import FIELD

KINDS = ("dens", "drvt", "hydro", "grav")
_EPI = {"dens": T.EPI_DENS, "drvt": T.EPI_DRVT, "hydro": T.EPI_HYDRO, "grav": T.EPI_GRAV}
_EPJ = {"dens": T.EPJ_DENS, "drvt": T.EPJ_DRVT, "hydro": T.EPJ_HYDRO, "grav": T.EPJ_GRAV}
_RES = {"dens": T.RES_DENS, "drvt": T.RES_DRVT, "hydro": T.RES_HYDRO, "grav": T.RES_GRAV}


def _payloads(S, ids):
    """EPI and EPJ records of every particle of the sorted state S (field-major)"""
    f = lambda k: S[FIELD[k]]
    pos = np.stack([f("x"), f("y"), f("z")], 1)
    vel = np.stack([f("vx"), f("vy"), f("vz")], 1)
    n = S.shape[1]
    epi, epj = {k: np.zeros(n, _EPI[k]) for k in KINDS}, {k: np.zeros(n, _EPJ[k]) for k in KINDS}
    for a in (epi["dens"], epj["dens"]):
        a["pos"], a["mass"], a["smth"] = pos, f("mass"), f("smth")
    epi["dens"]["id"] = ids
    for a in (epi["drvt"], epj["drvt"]):
        a["pos"], a["vel"], a["smth"] = pos, vel, f("smth")
    epi["drvt"]["dens"] = f("dens")
    epj["drvt"]["mass"] = f("mass")
    for a in (epi["hydro"], epj["hydro"]):
        a["pos"], a["vel"] = pos, vel
        for k in ("smth", "dens", "pres", "snds", "grad_smth"):
            a[k] = f(k)
        a["Bal"], a["AVa"], a["id"] = f("bal"), f("ava"), ids
    epj["hydro"]["mass"] = f("mass")
    epi["grav"]["pos"], epi["grav"]["eps2"], epi["grav"]["id"] = pos, f("smth") ** 2, ids   # class.h:336
    epj["grav"]["pos"], epj["grav"]["mass"], epj["grav"]["id"] = pos, f("mass"), ids
    return epi, epj


def _sph_lists(pos, h, start, count, q_large=0.995):
    """per group: the gather and symmetric superset j-lists (ascending sorted indices), as flat
    arrays with offsets.  A j belongs to the symmetric list when its distance to the group's box is
    below max(2.5 h_max of the group, 2.5 h_j): the candidates within 2.5 max(h_max, h_cut) of the
    box hold every such j with h_j <= h_cut (h_cut: the q_large quantile of h), and the few
    particles above h_cut are tested against every box, so the list is complete."""
    from scipy.spatial import cKDTree
    tree = cKDTree(pos)
    h_cut = float(np.quantile(h, q_large)) if len(h) else 0.0
    big = np.flatnonzero(h > h_cut)
    pb, rb = pos[big], 2.5 * h[big]
    gi, go, si, so = [], [0], [], [0]
    for s, c in zip(start, count):
        p = pos[s:s + c]
        lo, hi = p.min(0), p.max(0)
        ctr, half = 0.5 * (lo + hi), 0.5 * float(np.linalg.norm(hi - lo))
        hg = 2.5 * float(h[s:s + c].max())
        cand = np.asarray(tree.query_ball_point(ctr, half + max(hg, 2.5 * h_cut)), np.int64)
        cand.sort()
        d = np.sqrt((np.maximum(np.maximum(lo - pos[cand], pos[cand] - hi), 0.0) ** 2).sum(1))   # to the box
        g = cand[d < hg]
        sy = cand[d < np.maximum(hg, 2.5 * h[cand])]
        if len(big):
            db = np.sqrt((np.maximum(np.maximum(lo - pb, pb - hi), 0.0) ** 2).sum(1))
            extra = big[db < rb]
            if len(extra):
                sy = np.union1d(sy, extra)
        gi.append(g)
        si.append(sy)
        go.append(go[-1] + len(g))
        so.append(so[-1] + len(sy))
    return (np.concatenate(gi) if gi else np.zeros(0, np.int64), np.asarray(go, np.int64),
            np.concatenate(si) if si else np.zeros(0, np.int64), np.asarray(so, np.int64))


class Walks:
    """Walks of every gravity group of a context's current state (an FP64 context after a
    prologue or a step, so its gravity lists exist), ready for the batch entry points."""

    def __init__(self, ctx):
        from scipy.spatial import cKDTree  # noqa: F401  (fail early without scipy)
        F, ids_up, _ = ctx.download()
        slot, _ = ctx.order()
        S = F[:, slot]
        ids = ids_up[slot]
        self.n = S.shape[1]
        gl = ctx.grav_lists()
        tr = ctx.tree()
        self.start, self.count = gl["start"].astype(np.int64), gl["count"].astype(np.int64)
        self.n_group = len(self.start)
        epi, epj = _payloads(S, ids)
        pos = np.stack([S[FIELD[c]] for c in "xyz"], 1)
        g_idx, g_off, s_idx, s_off = _sph_lists(pos, S[FIELD["smth"]], self.start, self.count)
        self.epi = epi
        self.jlist = {"dens": (epj["dens"][g_idx], g_off), "drvt": (epj["drvt"][g_idx], g_off),
                      "hydro": (epj["hydro"][s_idx], s_off),
                      "grav": (epj["grav"][gl["epj"]], np.concatenate([gl["epj_off"], [len(gl["epj"])]]))}
        spj = np.zeros(len(gl["spj"]), T.SPJ_MONO)
        com = tr["com"][gl["spj"]]
        spj["pos"], spj["mass"] = com[:, :3], com[:, 3]
        self.spj = (spj, np.concatenate([gl["spj_off"], [len(gl["spj"])]]))
        # the index form: the whole EPJ array of each kind (every particle, sorted order), every cell
        # as an SPJ, and the walks' j entries as int32 indices into them
        self.epj_all = epj
        spj_all = np.zeros(len(tr["com"]), T.SPJ_MONO)
        spj_all["pos"], spj_all["mass"] = tr["com"][:, :3], tr["com"][:, 3]
        self.spj_all = spj_all
        i32 = lambda a: np.ascontiguousarray(a, dtype=np.int32)
        self.jindex = {"dens": (i32(g_idx), g_off), "drvt": (i32(g_idx), g_off), "hydro": (i32(s_idx), s_off),
                       "grav": (i32(gl["epj"]), self.jlist["grav"][1])}
        self.sindex = (i32(gl["spj"]), self.spj[1])
        self.result = {k: np.zeros(self.n, _RES[k]) for k in KINDS}
        self.staged_bytes = {k: self.n * _EPI[k].itemsize + len(self.jlist[k][0]) * _EPJ[k].itemsize
                             for k in KINDS}
        self.staged_bytes["grav"] += len(spj) * T.SPJ_MONO.itemsize
        # index form: EPI payloads, 4-byte indices, and the sent arrays once per pass
        self.index_bytes = {k: self.n * _EPI[k].itemsize + 4 * len(self.jindex[k][0]) + self.n * _EPJ[k].itemsize
                            for k in KINDS}
        self.index_bytes["grav"] += 4 * len(self.sindex[0]) + len(spj_all) * T.SPJ_MONO.itemsize
        self.sorted_state = S
        self._batch_cache = {}

    def _ptrs(self, arr, offs, w0, w1, itemsize):
        base = arr.ctypes.data
        return (C.c_void_p * (w1 - w0))(*[base + int(o) * itemsize for o in offs[w0:w1]])

    def _batches(self, kind, n_walk_limit, index=False):
        """the argument arrays of every batch of `kind` (walk pointers into this object's payload,
        index and result arrays, which stay in place, and the walk sizes), built once per (kind,
        n_walk_limit, form): FDPS hands its callbacks such arrays, so building them is not the
        boundary's cost"""
        key = (kind, n_walk_limit, index)
        if key not in self._batch_cache:
            epi = self.epi[kind]
            ej, jo = self.jindex[kind] if index else self.jlist[kind]
            res = self.result[kind]
            out = []
            for w0 in range(0, self.n_group, n_walk_limit):
                w1 = min(w0 + n_walk_limit, self.n_group)
                nw = w1 - w0
                args = [nw, self._ptrs(epi, self.start, w0, w1, epi.itemsize),
                        (C.c_int * nw)(*self.count[w0:w1].tolist()),
                        self._ptrs(ej, jo, w0, w1, ej.itemsize),
                        (C.c_int * nw)(*(jo[w0 + 1:w1 + 1] - jo[w0:w1]).tolist())]
                if kind == "grav":
                    sa, so = self.sindex if index else self.spj
                    args += [self._ptrs(sa, so, w0, w1, sa.itemsize),
                             (C.c_int * nw)(*(so[w0 + 1:w1 + 1] - so[w0:w1]).tolist())]
                if index:   # the sent arrays (used by the send call only) and send_flag = 0
                    ea = self.epj_all[kind]
                    args += [ea.ctypes.data, len(ea)]
                    if kind == "grav":
                        args += [self.spj_all.ctypes.data, len(self.spj_all)]
                    args += [0]
                out.append((args, self._ptrs(res, self.start, w0, w1, res.itemsize)))
            self._batch_cache[key] = out
        return self._batch_cache[key]

    def run(self, kind, n_walk_limit=256, n_tags=4, tag0=0, index=False):
        """one pass of `kind` over every walk, the MultiWalk way (index: the index form, whose first
        call sends the pass's EPJ / SPJ arrays); returns the host seconds taken"""
        from . import lib
        L = lib.load()
        res = self.result[kind]
        res[:] = np.zeros(1, _RES[kind])
        if kind == "grav":
            res["dt"] = 1.0e30   # RESULT::Grav::clear()
        batches = self._batches(kind, n_walk_limit, index)
        disp = getattr(L, f"sph_dispatch_index_{kind}" if index else f"sph_dispatch_{kind}")
        retr = getattr(L, f"sph_retrieve_{kind}")
        pend = {}

        def retrieve(tag):
            args, rp = pend.pop(tag)
            rc = retr(tag0 + tag, args[0], args[2], rp)
            if rc != 0:
                raise lib.SphError(rc, L.sph_batch_last_error().decode())

        t0 = time.perf_counter()
        if index and batches:   # the send call: no walks, the whole arrays, send_flag = 1
            a0 = batches[0][0]
            none = [0, None, None, None, None] + ([None, None] if kind == "grav" else [])   # no walks
            rc = disp(tag0, *none, *a0[len(none):-1], 1)
            if rc != 0:
                raise lib.SphError(rc, L.sph_batch_last_error().decode())
        for b, (args, rp) in enumerate(batches):
            tag = b % n_tags
            if tag in pend:
                retrieve(tag)
            rc = disp(tag0 + tag, *args)
            if rc != 0:
                raise lib.SphError(rc, L.sph_batch_last_error().decode())
            pend[tag] = (args, rp)
        for tag in list(pend):
            retrieve(tag)
        return time.perf_counter() - t0

    def step(self, n_dens_iter=4, **kw):   # kw: n_walk_limit, n_tags, tag0, index
        """the functor calls of one step of main.cpp:136-147 (density x n_dens_iter, derivative,
        hydro, gravity) on these walks; the seconds of each pass"""
        out = {"dens": sum(self.run("dens", **kw) for _ in range(n_dens_iter))}
        for k in ("drvt", "hydro", "grav"):
            out[k] = self.run(k, **kw)
        return out
