"""Snapshots and checkpoints of the particle state.

* Text snapshots in the reference's format: FDPS ``writeParticleAscii`` of
  ``RealPtcl`` (class.h:173-180, header class.h:21-30, file naming and call
  io.h:28-47): a file ``<base>_<nproc>_<rank>.dat`` holding the time (``%e``)
  and the particle count (``%d``) on two lines, then one line per particle,
  tab-separated, ``id tag mass x y z vx vy vz dens eng pres pot ent temp``
  (``%lld`` / ``%lf``).  ``tag`` carries the material slot; ``ent`` and
  ``temp`` are the state's entropy and temperature (written by mode 2).
  The format rounds to 6 decimals, as the reference's does.
* Checkpoints: a pointer-free binary file that restores a context exactly
  (the reference's restart file, io.h:7-23, writes raw structs including an
  EoS pointer).  Layout: the 8-byte magic ``SPHGB3CK``, a little-endian
  uint64 header length, a JSON header (format version, field names, per-run
  particle counts, times, dts, steps, and the byte offsets of the arrays),
  then per run the field-major float64 state [34][n], int64 ids and int32
  material slots.  Restored with forces valid, so the next step continues
  the same trajectory.
"""
import json
import os
import struct

import numpy as np

from .ic import FIELD, FIELDS, NFIELD

ASCII_COLUMNS = ["id", "tag", "mass", "x", "y", "z", "vx", "vy", "vz", "dens", "eng", "pres", "pot", "ent", "temp"]
MAGIC = b"SPHGB3CK"
VERSION = 2   # 2: the state carries ent and temp (34 fields)


def ascii_path(base: str, nproc: int = 1, rank: int = 0) -> str:
    """FDPS's file name for one rank's part of a snapshot (format "%s_%05d_%05d.dat")"""
    return "%s_%05d_%05d.dat" % (base, nproc, rank)


def write_ascii(base: str, F: np.ndarray, ids: np.ndarray, mats: np.ndarray, time: float) -> str:
    """writes one snapshot in the reference's text format; returns the file name"""
    n = F.shape[1]
    path = ascii_path(base)
    cols = [F[FIELD[c]] for c in ASCII_COLUMNS[2:]]
    with open(path, "w") as fh:
        fh.write("%e\n%d\n" % (time, n))
        fmt = "%d\t%d\t" + "\t".join(["%f"] * len(cols)) + "\n"
        for i in range(n):
            fh.write(fmt % ((int(ids[i]), int(mats[i])) + tuple(float(c[i]) for c in cols)))
    return path


def read_ascii(path: str):
    """reads a snapshot in the reference's text format: (F [32][n] with the columns it holds, ids, tags, time)"""
    with open(path) as fh:
        time = float(fh.readline())
        n = int(fh.readline())
        rows = np.loadtxt(fh, ndmin=2) if n > 0 else np.zeros((0, len(ASCII_COLUMNS)))
    if rows.shape[0] != n:
        raise ValueError(f"{path}: header says {n} particles, found {rows.shape[0]}")
    F = np.zeros((NFIELD, n))
    for k, c in enumerate(ASCII_COLUMNS[2:], start=2):
        if c in FIELD:
            F[FIELD[c]] = rows[:, k]
    return F, rows[:, 0].astype(np.int64), rows[:, 1].astype(np.int32), time


def _runs_of(ctx):
    out = []
    for h in ctx.runs():
        info = ctx.run_info(h)
        F, ids, mats = ctx.download_run(h)
        out.append((info, F, ids, mats))
    return out


def write_checkpoint(path: str, ctx) -> None:
    """every run of a context, with its time, dt and step count"""
    runs = _runs_of(ctx)
    header = {"format": "fdps_sph_gb300 checkpoint", "version": VERSION, "fields": list(FIELDS), "runs": []}
    off = 0
    for info, F, ids, mats in runs:
        n = F.shape[1]
        header["runs"].append({"n": n, "time": info["time"], "dt": info["dt"], "steps": info["steps"],
                               "state": off, "ids": off + 8 * NFIELD * n, "materials": off + 8 * NFIELD * n + 8 * n})
        off += 8 * NFIELD * n + 8 * n + 4 * n
    hb = json.dumps(header).encode()
    with open(path, "wb") as fh:
        fh.write(MAGIC)
        fh.write(struct.pack("<Q", len(hb)))
        fh.write(hb)
        for info, F, ids, mats in runs:
            fh.write(np.ascontiguousarray(F, "<f8").tobytes())
            fh.write(np.ascontiguousarray(ids, "<i8").tobytes())
            fh.write(np.ascontiguousarray(mats, "<i4").tobytes())


def read_checkpoint(path: str):
    """[(F, ids, mats, info)] per run"""
    with open(path, "rb") as fh:
        if fh.read(8) != MAGIC:
            raise ValueError(f"{path} is not a checkpoint")
        hl = struct.unpack("<Q", fh.read(8))[0]
        header = json.loads(fh.read(hl))
        if header.get("version") != VERSION or header.get("fields") != list(FIELDS):
            raise ValueError(f"{path}: unsupported checkpoint version or field layout")
        data = fh.read()
    out = []
    for r in header["runs"]:
        n = r["n"]
        F = np.frombuffer(data, "<f8", NFIELD * n, r["state"]).reshape(NFIELD, n).copy()
        ids = np.frombuffer(data, "<i8", n, r["ids"]).copy()
        mats = np.frombuffer(data, "<i4", n, r["materials"]).copy()
        out.append((F, ids, mats, {k: r[k] for k in ("time", "dt", "steps")}))
    return out


def restore(ctx, path: str):
    """adds every run of a checkpoint to a context (forces valid: the next step continues each
    run; step counters restart at 0); returns the new run handles"""
    hs = []
    for F, ids, mats, info in read_checkpoint(path):
        hs.append(ctx.add_run(F, ids, mats, time=info["time"], dt=info["dt"], forces_valid=info["dt"] > 0.0))
    return hs


def restore_single(ctx, path: str):
    """a one-run checkpoint into a context made by upload (the sph_upload / sph_step API)"""
    runs = read_checkpoint(path)
    if len(runs) != 1:
        raise ValueError(f"{path} holds {len(runs)} runs")
    F, ids, mats, info = runs[0]
    ctx.upload(F, ids, mats, time=info["time"], dt=info["dt"], forces_valid=info["dt"] > 0.0)
    return info


if __name__ == "__main__":   # pragma: no cover
    import sys
    F, ids, tags, t = read_ascii(sys.argv[1])
    print(os.path.basename(sys.argv[1]), "time", t, "particles", F.shape[1])
