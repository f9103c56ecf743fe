"""Generates the golden fixtures under tests/golden/ by running the
reference's own physics code (oracle/_ref/ref_driver: the reference headers
compiled unmodified against oracle/ref/ps_shim.hpp).

Run here, where the reference sources exist:
    python tests/golden/make_golden.py

Fixtures (npz):
  kernel.npz      W / gradW samples (kernel.h:8-34)
  eos_small.npz   bilinear lookups on a small synthetic rho-u table through
                  the reference's ANEOS and Tillotson classes (EoS.h:241-247,
                  394-400; interpolation.h:33-102), incl. edge / outside points
  eos_dunite200.npz  lookups on the 200 x 200 synthetic dunite table
  functors.npz    CalcDensity / CalcDerivative (+Balsara) / CalcHydroForce /
                  CalcGravityForce outputs on a seeded 700-particle body,
                  with FDPS-style group-superset walks and exact-list walks
  integ.npz       initialKick/fullDrift/predict/finalKick/dampMotion records
  dtglobal.npz    getTimeStepGlobal
  eos_mode2.npz   the mode-2 EoS surface: InternalEnergy(rho, s)
                  (RestrictedBilinearInterpolation, interpolation.h:107-335),
                  Temperature and Entropy (EoS.h:249-260, 402-413) through the
                  reference's ANEOS class, on a 120 x 120 synthetic table, a
                  12 x 120 table with sub-unit entropy steps (where the
                  int abs(int) of the reference's translation unit and a
                  floating abs pick different neighbours; both builds of the
                  driver are run) and the 200 x 200 synthetic dunite table;
                  plus points where the reference's lookup is undefined or
                  not finite (checked against the oracle only)
  tillotson.npz   the analytic branches P_co / P_ex of the reference's
                  Tillotson class (EoS.h:91-103, private and never called by
                  the reference; read through the driver's explicit-
                  instantiation access) with the granite (EoS.h:446) and iron
                  (EoS.h:448) parameters, on compressed, cold-expanded,
                  hot-expanded and blend-region points
The particle state, the walks (group ranges and j indices) and the reference
outputs are stored; tables are regenerated from their stored parameters.
"""
from __future__ import annotations

import os
import struct
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)

from fdps_sph_gb300 import eos, ic, layouts as T  # noqa: E402
from oracle import build_oracle, pyoracle as po  # noqa: E402

REF_ROOT = build_oracle.REF_ROOT
DRIVER = os.path.join(ROOT, "oracle", "_ref", "ref_driver")
DRIVER_FABS = os.path.join(ROOT, "oracle", "_ref", "ref_driver_fabs")


def run_ref(mode: str, payload: bytes, n_out_bytes: int | None = None, driver: str = DRIVER) -> bytes:
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fi, "wb") as fh:
            fh.write(payload)
        subprocess.run([driver, mode, fi, fo], check=True, cwd=REF_ROOT)
        with open(fo, "rb") as fh:
            out = fh.read()
    if n_out_bytes is not None and len(out) != n_out_bytes:
        raise RuntimeError(f"{mode}: got {len(out)} bytes, expected {n_out_bytes}")
    return out


# ---------------------------------------------------------------------------
def gen_kernel(rng):
    h = 10.0 ** rng.uniform(-2, 6, 400)
    r = h * 2.5 * rng.uniform(0, 1.2, 400)
    d = rng.normal(size=(400, 3))
    d /= np.linalg.norm(d, axis=1)[:, None]
    dr = d * r[:, None]
    dr[:8] = 0.0                                   # r = 0 (self term)
    dr[8:16, 0] = 2.5 * h[8:16]                    # exactly at the support radius
    rec = np.concatenate([dr, h[:, None]], axis=1)
    out = run_ref("kernel", struct.pack("<i", len(rec)) + rec.astype("<f8").tobytes())
    o = np.frombuffer(out, dtype="<f8").reshape(-1, 4)
    np.savez_compressed(os.path.join(HERE, "kernel.npz"), dr=dr, h=h, W=o[:, 0], gradW=o[:, 1:4])


def _eos_payload(path, kind, pts):
    pb = path.encode()
    return (struct.pack("<i", len(pb)) + pb + struct.pack("<ii", kind, len(pts)) +
            np.ascontiguousarray(pts, dtype="<f8").tobytes())


def _eos_points(rng, t: eos.Table, n_rand=600):
    rho, u = t.rho, t.u
    lr = np.log(rho[0]), np.log(rho[-1])
    lu = np.log(u[0]), np.log(u[-1])
    pts = [np.stack([np.exp(rng.uniform(lr[0] - 0.5, lr[1] + 0.5, n_rand)),
                     np.exp(rng.uniform(lu[0] - 0.5, lu[1] + 0.5, n_rand))], axis=1)]
    # exact grid nodes, interval midpoints, first / last intervals, outside
    ii = rng.integers(0, len(rho), 60)
    jj = rng.integers(0, len(u), 60)
    pts.append(np.stack([rho[ii], u[jj]], axis=1))
    mi = rng.integers(0, len(rho) - 1, 60)
    mj = rng.integers(0, len(u) - 1, 60)
    pts.append(np.stack([0.5 * (rho[mi] + rho[mi + 1]), 0.5 * (u[mj] + u[mj + 1])], axis=1))
    pts.append(np.array([[0.5 * (rho[0] + rho[1]), u[len(u) // 2]], [0.5 * (rho[-2] + rho[-1]), u[len(u) // 2]],
                         [rho[len(rho) // 2], 0.5 * (u[0] + u[1])], [rho[len(rho) // 2], 0.5 * (u[-2] + u[-1])],
                         [rho[0] * 0.1, u[3]], [rho[-1] * 10, u[3]], [rho[3], u[0] * 0.1], [rho[3], u[-1] * 10],
                         [0.0, 0.0], [-1.0, 1e5]]))
    return np.concatenate(pts)


def gen_eos(rng):
    small = eos.synthetic_table("iron", n_rho=30, n_u=25, rho_range=(1e2, 3e4), u_range=(1e4, 1e9))
    big = eos.synthetic_table("dunite")
    for name, t, spec in [("eos_small.npz", small, dict(material="iron", n_rho=30, n_u=25, rho_range=(1e2, 3e4),
                                                                  u_range=(1e4, 1e9))),
                          ("eos_dunite200.npz", big, dict(material="dunite", n_rho=200, n_u=200,
                                                          rho_range=(1e1, 3e4), u_range=(1e3, 1e9)))]:
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "t.rho_u.txt")
            eos.write_rho_u(path, t)
            back = eos.read_rho_u(path)
            assert np.array_equal(back.pres, t.pres) and np.array_equal(back.rho, t.rho)
            pts = _eos_points(rng, t)
            outs = {}
            for kind, label in [(0, "aneos"), (1, "tillotson_table")]:
                o = run_ref("eos_file", _eos_payload(path, kind, pts))
                outs[label] = np.frombuffer(o, dtype="<f8").reshape(-1, 2)
        np.savez_compressed(os.path.join(HERE, name), points=pts, P=outs["aneos"][:, 0], cs=outs["aneos"][:, 1],
                            P_til=outs["tillotson_table"][:, 0], cs_til=outs["tillotson_table"][:, 1],
                            rho=t.rho, u=t.u, pres=t.pres, snds=t.snds,
                            spec=np.array(repr(spec)))


# ---------------------------------------------------------------------------
def golden_state(seed=77):
    """A 700-particle two-layer body with a rotating, expanding and noisy
    velocity field and perturbed smoothing lengths (so div v, curl v, AV and
    the Balsara switch are all non-trivial)."""
    rng = np.random.default_rng(seed)
    body = ic.Body(700, 1.0e23, [ic.Layer(0, 0.3, 7800.0), ic.Layer(1, 0.7, 2700.0)])
    F, mats, R = ic.make_body(body, rng)
    X = F[[ic.FIELD["x"], ic.FIELD["y"], ic.FIELD["z"]]].T
    omega = np.array([0.0, 0.0, 2.0e-4])
    V = np.cross(omega, X) + 1.0e-4 * X + rng.normal(scale=50.0, size=X.shape)
    for k, c in enumerate("xyz"):
        F[ic.FIELD["v" + c]] = V[:, k]
    F[ic.FIELD["smth"]] *= rng.uniform(0.9, 1.15, F.shape[1])
    F[ic.FIELD["eng"]] = 1.0e6 * rng.uniform(0.5, 2.0, F.shape[1])
    ids = np.arange(F.shape[1], dtype=np.int64)
    return F, ids, mats


def _superset_walks(F, cells, groups, h_of):
    """FDPS Gather-style walks: the group's i-particles and every particle
    within the group's bounding box inflated by the group's largest search
    radius (so the j-list is a superset of every i's neighbours)."""
    x, y, z = F[ic.FIELD["x"]], F[ic.FIELD["y"]], F[ic.FIELD["z"]]
    P = np.stack([x, y, z], axis=1)
    walks = []
    for g in groups:
        c = cells[g]
        s, n = int(c["start"]), int(c["count"])
        lo, hi = P[s:s + n].min(axis=0), P[s:s + n].max(axis=0)
        R = 2.5 * h_of[s:s + n].max()
        d = np.maximum(np.maximum(lo - P, P - hi), 0.0)
        js = np.nonzero((d * d).sum(axis=1) <= R * R)[0].astype(np.int32)
        walks.append((s, n, js))
    return walks


def _walk_bytes(walks, epi_fn, epj_fn, spj=None):
    b = [struct.pack("<i", len(walks))]
    for k, (s, n, js) in enumerate(walks):
        ns = 0 if spj is None else len(spj[k])
        b.append(struct.pack("<iii", n, len(js), ns))
        b.append(epi_fn(np.arange(s, s + n)).tobytes())
        b.append(epj_fn(js).tobytes())
        if ns:
            b.append(spj[k].tobytes())
    return b"".join(b)


def _pack_walks(walks):
    starts = np.array([w[0] for w in walks], dtype=np.int32)
    counts = np.array([w[1] for w in walks], dtype=np.int32)
    joff = np.zeros(len(walks) + 1, dtype=np.int64)
    joff[1:] = np.cumsum([len(w[2]) for w in walks])
    jidx = np.concatenate([w[2] for w in walks]).astype(np.int32) if walks else np.zeros(0, np.int32)
    return starts, counts, joff, jidx


def gen_functors():
    F, ids, mats = golden_state()
    mset = po.MaterialSet([eos.Tillotson("iron", eos.TILLOTSON["iron"]).as_material(),
                           eos.Tillotson("granite", eos.TILLOTSON["granite"]).as_material()])
    cfg = po.make_config(mset)
    s = po.OracleSystem(F, ids, mats)
    tr = po.OracleTree(s, 8)          # sorts s into key order
    cells = tr.cells()
    sph_groups = tr.groups(128)
    out = {}
    G = lambda name: s.field(name)    # noqa: E731

    # ---- density: state before the pass, reference result -------------------
    F0 = s.F.copy()
    out["state_dens"] = F0
    wd = _superset_walks(F0, cells, sph_groups, F0[ic.FIELD["smth"]])

    def epi_dens(idx):
        a = np.zeros(len(idx), T.EPI_DENS)
        a["pos"] = F0[[0, 1, 2]][:, idx].T
        a["mass"] = F0[ic.FIELD["mass"], idx]
        a["smth"] = F0[ic.FIELD["smth"], idx]
        a["id"] = s.id[idx]
        return a

    def epj_dens(idx):
        a = np.zeros(len(idx), T.EPJ_DENS)
        a["pos"] = F0[[0, 1, 2]][:, idx].T
        a["mass"] = F0[ic.FIELD["mass"], idx]
        a["smth"] = F0[ic.FIELD["smth"], idx]
        return a

    r = np.frombuffer(run_ref("dens", _walk_bytes(wd, epi_dens, epj_dens)), dtype=T.RES_DENS)
    out["dens_walks"] = _pack_walks(wd)
    out["ref_dens"] = r.copy()

    # advance the state with the oracle: density x4, pressure
    for _ in range(4):
        tr.pass_density(cfg)
    tr.pass_pressure(cfg)
    # the tree's hmax must follow the new h for the symmetric walk: rebuild (positions unchanged -> same order)
    tr = po.OracleTree(s, 8)
    cells = tr.cells()
    sph_groups = tr.groups(128)
    F1 = s.F.copy()
    out["state_drvt"] = F1
    wv = _superset_walks(F1, cells, sph_groups, F1[ic.FIELD["smth"]])

    def epi_drvt(idx):
        a = np.zeros(len(idx), T.EPI_DRVT)
        a["pos"] = F1[[0, 1, 2]][:, idx].T
        a["vel"] = F1[[3, 4, 5]][:, idx].T
        a["smth"] = F1[ic.FIELD["smth"], idx]
        a["dens"] = F1[ic.FIELD["dens"], idx]
        return a

    def epj_drvt(idx):
        a = np.zeros(len(idx), T.EPJ_DRVT)
        a["mass"] = F1[ic.FIELD["mass"], idx]
        a["pos"] = F1[[0, 1, 2]][:, idx].T
        a["vel"] = F1[[3, 4, 5]][:, idx].T
        a["smth"] = F1[ic.FIELD["smth"], idx]
        return a

    r = np.frombuffer(run_ref("drvt", _walk_bytes(wv, epi_drvt, epj_drvt)), dtype=T.RES_DRVT)
    out["drvt_walks"] = _pack_walks(wv)
    out["ref_drvt"] = r.copy()
    # Balsara switch through RealPtcl::copyFromForce (class.h:132-142)
    n = s.n
    rec = np.zeros((n, 7))
    rec[:, 0] = r["div_v"]
    rec[:, 1:4] = r["rot_v"]
    rec[:, 4] = r["grad_smth"]
    rec[:, 5] = F1[ic.FIELD["snds"]]
    rec[:, 6] = F1[ic.FIELD["smth"]]
    b = np.frombuffer(run_ref("balsara", struct.pack("<i", n) + rec.astype("<f8").tobytes()),
                      dtype="<f8").reshape(-1, 3)
    out["ref_bal"] = b[:, 0].copy()

    tr.pass_derivative()
    F2 = s.F.copy()
    out["state_hydro"] = F2
    hmax_w = F2[ic.FIELD["smth"]].max()
    # symmetric superset: inflate by the largest search radius anywhere
    wh = _superset_walks(F2, cells, sph_groups, np.full(n, hmax_w))

    def epi_hydro(idx):
        a = np.zeros(len(idx), T.EPI_HYDRO)
        a["pos"] = F2[[0, 1, 2]][:, idx].T
        a["vel"] = F2[[3, 4, 5]][:, idx].T
        for k in ("smth", "dens", "pres", "snds", "grad_smth"):
            a[k] = F2[ic.FIELD[k], idx]
        a["Bal"] = F2[ic.FIELD["bal"], idx]
        a["AVa"] = F2[ic.FIELD["ava"], idx]
        a["id"] = s.id[idx]
        return a

    def epj_hydro(idx):
        a = np.zeros(len(idx), T.EPJ_HYDRO)
        a["pos"] = F2[[0, 1, 2]][:, idx].T
        a["vel"] = F2[[3, 4, 5]][:, idx].T
        for k in ("dens", "mass", "smth", "pres", "grad_smth", "snds"):
            a[k] = F2[ic.FIELD[k], idx]
        a["Bal"] = F2[ic.FIELD["bal"], idx]
        a["AVa"] = F2[ic.FIELD["ava"], idx]
        a["id"] = s.id[idx]
        return a

    r = np.frombuffer(run_ref("hydro", _walk_bytes(wh, epi_hydro, epj_hydro)), dtype=T.RES_HYDRO)
    out["hydro_walks"] = _pack_walks(wh)
    out["ref_hydro_superset"] = r.copy()
    # exact symmetric lists, one walk per particle (the list semantics the device implements)
    we = [(i, 1, tr.sph_list(i, 1)) for i in range(n)]
    r = np.frombuffer(run_ref("hydro", _walk_bytes(we, epi_hydro, epj_hydro)), dtype=T.RES_HYDRO)
    out["hydro_exact_walks"] = _pack_walks(we)
    out["ref_hydro_exact"] = r.copy()

    # ---- gravity: oracle groups / lists, reference functors -----------------
    ggroups = tr.groups(256)
    wg, spjs = [], []
    for g in ggroups:
        epj, spj = tr.grav_list(int(g), 0.5)
        c = cells[g]
        wg.append((int(c["start"]), int(c["count"]), epj))
        sp = np.zeros(len(spj), T.SPJ_MONO)
        sp["mass"] = cells["mass"][spj]
        sp["pos"] = np.stack([cells["com"][spj, 0], cells["com"][spj, 1], cells["com"][spj, 2]], axis=1)
        spjs.append(sp)

    def epi_grav(idx):
        a = np.zeros(len(idx), T.EPI_GRAV)
        a["pos"] = F2[[0, 1, 2]][:, idx].T
        a["eps2"] = F2[ic.FIELD["smth"], idx] ** 2
        a["id"] = s.id[idx]
        return a

    def epj_grav(idx):
        a = np.zeros(len(idx), T.EPJ_GRAV)
        a["pos"] = F2[[0, 1, 2]][:, idx].T
        a["mass"] = F2[ic.FIELD["mass"], idx]
        a["id"] = s.id[idx]
        return a

    r = np.frombuffer(run_ref("grav", _walk_bytes(wg, epi_grav, epj_grav, spjs)), dtype=T.RES_GRAV)
    out["grav_walks"] = _pack_walks(wg)
    spj_off = np.zeros(len(spjs) + 1, dtype=np.int64)
    spj_off[1:] = np.cumsum([len(a) for a in spjs])
    out["grav_spj"] = np.concatenate(spjs) if spjs else np.zeros(0, T.SPJ_MONO)
    out["grav_spj_off"] = spj_off
    out["ref_grav"] = r.copy()

    flat = {}
    for k, v in out.items():
        if k.endswith("_walks"):
            flat[k + "_start"], flat[k + "_count"], flat[k + "_joff"], flat[k + "_jidx"] = v
        else:
            flat[k] = v
    flat["ids"] = s.id.copy()
    flat["mats"] = s.mat.copy()
    np.savez_compressed(os.path.join(HERE, "functors.npz"), **flat)


def gen_integ(rng):
    n = 200
    rec = rng.normal(size=(n, 21)) * np.array([1e7] * 3 + [1e3] * 3 + [1.0] * 6 + [1e6, 1e3] + [1.0] * 6 + [1e3])
    dt, damping = 17.25, 0.999
    payload = struct.pack("<i", n) + struct.pack("<dd", dt, damping) + rec.astype("<f8").tobytes()
    o = np.frombuffer(run_ref("integ", payload), dtype="<f8").reshape(n, 15)
    np.savez_compressed(os.path.join(HERE, "integ.npz"), rec=rec, dt=dt, damping=damping, out=o)
    n2 = 500
    r2 = np.abs(rng.normal(size=(n2, 7))) * 10 + 0.1
    dtv = np.frombuffer(run_ref("dtglobal", struct.pack("<i", n2) + r2.astype("<f8").tobytes()), dtype="<f8")
    np.savez_compressed(os.path.join(HERE, "dtglobal.npz"), rec=r2, dt=dtv[0])


def fine_entropy_table():
    """12 x 120 table whose entropy rises by 0.6 per energy column: nearest-entropy
    distances below 1 truncate to 0 under int abs(int)"""
    rho = np.array([float("%15.8E" % v) for v in np.geomspace(1.0e2, 2.0e4, 12)])
    u = np.array([float("%15.8E" % v) for v in np.geomspace(1.0e4, 1.0e8, 120)])
    R, U = np.meshgrid(rho, u, indexing="ij")
    P, cs = eos.tillotson_eval(eos.TILLOTSON["iron"], R, U)
    r8 = np.vectorize(lambda v: float("%15.8E" % v))
    ent = r8(3000.0 + 0.6 * np.arange(120)[None, :] + 0.05 * np.arange(12)[:, None])
    return eos.Table(rho=rho, u=u, pres=r8(P), snds=r8(cs), temp=r8(U / 1.0e3), ent=ent, name="fine-entropy")


def mode2_tables():
    """(name, table, spec) of the mode-2 fixture; spec rebuilds a synthetic table"""
    out = []
    spec = dict(material="iron", n_rho=120, n_u=120, rho_range=(1e-3, 3e4), u_range=(1e3, 1e9))
    out.append(("iron120", eos.synthetic_table(**spec), spec))
    out.append(("fine", fine_entropy_table(), None))
    spec = dict(material="dunite", n_rho=200, n_u=200, rho_range=(1e1, 3e4), u_range=(1e3, 1e9))
    out.append(("dunite200", eos.synthetic_table(**spec), spec))
    return out


def _mode2_points(rng, t: eos.Table, n=500):
    lr = np.log(t.rho[1]), np.log(t.rho[-2])
    lu = np.log(t.u[1]), np.log(t.u[-2])
    e = t.ent.reshape(-1)
    rho = np.exp(rng.uniform(*lr, n))
    s = rng.uniform(np.percentile(e, 5), np.percentile(e, 95), n)
    u = np.exp(rng.uniform(*lu, n))
    return np.stack([rho, s, u], 1)


def _mode2_edges(rng, t: eos.Table):
    """points where the reference's lookup is NaN (density on a table row, below the
    table) or undefined (above the table, entropies outside the slices)"""
    e = t.ent.reshape(-1)
    rows = t.rho[rng.integers(1, len(t.rho) - 1, 8)]
    mid_s = float(np.median(e))
    pts = [[r, mid_s, t.u[3]] for r in rows]
    pts += [[t.rho[0] * 0.5, mid_s, t.u[3]], [t.rho[-1] * 2.0, mid_s, t.u[3]], [t.rho[-1], mid_s, t.u[3]],
            [np.sqrt(t.rho[3] * t.rho[4]), e.min() - 1.0e4, t.u[3]],
            [np.sqrt(t.rho[3] * t.rho[4]), e.max() + 1.0e4, t.u[3]],
            [np.sqrt(t.rho[3] * t.rho[4]), 3.0e9, t.u[3]], [np.nan, mid_s, t.u[3]]]
    return np.array(pts)


def gen_eos_mode2():
    rng = np.random.default_rng(120)
    out = {}
    for name, t, spec in mode2_tables():
        ms = po.MaterialSet([t.as_material()])
        pts = _mode2_points(rng, t)
        defined = np.ones(len(pts), bool)
        for k, (r, sv, _) in enumerate(pts):
            for am in (0, 1):
                v, undef = ms.internal_energy(0, r, sv, 120, am)
                defined[k] &= (not undef) and bool(np.isfinite(v))
        pts = pts[defined]
        with tempfile.TemporaryDirectory() as td:
            path = os.path.join(td, "t.rho_u.txt")
            eos.write_rho_u(path, t)
            back = eos.read_rho_u(path)
            assert np.array_equal(back.ent, t.ent) and np.array_equal(back.temp, t.temp)
            pb = path.encode()
            payload = (struct.pack("<i", len(pb)) + pb + struct.pack("<iii", 0, 120, len(pts)) +
                       np.ascontiguousarray(pts, "<f8").tobytes())
            o_int = np.frombuffer(run_ref("eos_mode2", payload), "<f8").reshape(-1, 3)
            o_real = np.frombuffer(run_ref("eos_mode2", payload, driver=DRIVER_FABS), "<f8").reshape(-1, 3)
        out[f"{name}_points"] = pts
        out[f"{name}_U_int"] = o_int[:, 0]
        out[f"{name}_U_real"] = o_real[:, 0]
        out[f"{name}_T"] = o_int[:, 1]
        out[f"{name}_S"] = o_int[:, 2]
        out[f"{name}_edges"] = _mode2_edges(rng, t)
        out[f"{name}_spec"] = np.array(repr(spec))
        if spec is None:   # not a synthetic_table: store the table itself
            for f in ("rho", "u", "pres", "snds", "temp", "ent"):
                out[f"{name}_table_{f}"] = getattr(t, f)
        print(f"eos_mode2 {name}: {len(pts)} defined points, int/real abs differ at "
              f"{int(np.sum(o_int[:, 0] != o_real[:, 0]))}")
    np.savez_compressed(os.path.join(HERE, "eos_mode2.npz"), **out)


# region codes of tillotson.npz: which of the reference's branches a point's pressure takes
TIL_COMPRESSED, TIL_COLD, TIL_HOT, TIL_BLEND = 0, 1, 2, 3


def gen_tillotson(seed=20261204):
    """P_co and P_ex of the reference's Tillotson class (EoS.h:91-103) with the granite parameters
    (EoS.h:446) and the iron ones (EoS.h:448), on points of each region: compressed (rho >= rho0),
    cold expanded (rho < rho0, u <= uiv), hot expanded (rho < rho0, u >= ucv) and the blend region
    between them (rho < rho0, uiv < u < ucv).  The constructor reads the named table file, which
    does not enter the two branches."""
    rng = np.random.default_rng(seed)
    out = {}
    for name, path in (("granite", "eos/granite.rho_u.txt"), ("iron", "eos/iron___.rho_u.txt")):
        par = np.array(eos.TILLOTSON[name], dtype=np.float64)
        rho0, uiv, ucv = par[0], par[2], par[3]
        m = 150
        groups = [
            (TIL_COMPRESSED, rho0 * rng.uniform(1.0, 3.0, m), np.exp(rng.uniform(np.log(1e3), np.log(1e9), m))),
            (TIL_COLD, rho0 * rng.uniform(0.3, 1.0, m), rng.uniform(1e3, uiv, m)),
            (TIL_HOT, rho0 * rng.uniform(0.05, 1.0, m), np.exp(rng.uniform(np.log(ucv), np.log(1e9), m))),
            (TIL_BLEND, rho0 * rng.uniform(0.05, 1.0, m), rng.uniform(uiv, ucv, m)),
        ]
        # the region edges themselves: rho = rho0, u = uiv, u = ucv
        edge = [(TIL_COMPRESSED, np.full(4, rho0), np.array([1e3, uiv, ucv, 1e8])),
                (TIL_COLD, rho0 * np.array([0.5, 0.9]), np.full(2, uiv)),
                (TIL_HOT, rho0 * np.array([0.5, 0.9]), np.full(2, ucv))]
        region = np.concatenate([np.full(len(r), g, np.int32) for g, r, _ in groups + edge])
        rho = np.concatenate([r for _, r, _ in groups + edge])
        u = np.concatenate([v for _, _, v in groups + edge])
        pb = path.encode()
        payload = (par.astype("<f8").tobytes() + struct.pack("<i", len(pb)) + pb + struct.pack("<i", len(rho)) +
                   np.ascontiguousarray(np.stack([rho, u], 1), dtype="<f8").tobytes())
        o = np.frombuffer(run_ref("tillotson", payload), dtype="<f8").reshape(-1, 2)
        out.update({f"{name}_par": par, f"{name}_rho": rho, f"{name}_u": u, f"{name}_region": region,
                    f"{name}_P_co": o[:, 0].copy(), f"{name}_P_ex": o[:, 1].copy()})
    np.savez_compressed(os.path.join(HERE, "tillotson.npz"), **out)


GENERATORS = ("kernel", "eos", "functors", "integ", "eos_mode2", "tillotson")


def main(which=GENERATORS):
    build_oracle.build()
    if not os.path.exists(DRIVER):
        raise SystemExit("reference driver not built (reference sources absent?)")
    rng = np.random.default_rng(20261203)   # shared, in this order, by the first four generators
    if "kernel" in which:
        gen_kernel(rng)
    if "eos" in which:
        gen_eos(rng)
    if "functors" in which:
        gen_functors()
    if "integ" in which:
        gen_integ(rng)
    if "eos_mode2" in which:
        gen_eos_mode2()
    if "tillotson" in which:
        gen_tillotson()
    print("golden fixtures written to", HERE)


if __name__ == "__main__":
    # python tests/golden/make_golden.py [generator ...]   (default: all; a generator sharing the
    # first four's random stream regenerates only what it would have written in a full run when the
    # generators before it run too)
    main(tuple(sys.argv[1:]) or GENERATORS)
