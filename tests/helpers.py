"""Shared set-up for the parity tests: identical initial conditions and EoS
materials for the device library (C ABI) and the CPU oracle."""
from __future__ import annotations

import os

import numpy as np

from fdps_sph_gb300 import eos, ic

GOLD = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    return np.load(os.path.join(GOLD, name), allow_pickle=False)


def tillotson_materials():
    """material 0 = iron, 1 = granite (analytic Tillotson, EoS.h:446/448 parameters)."""
    return [eos.Tillotson("iron", eos.TILLOTSON["iron"]), eos.Tillotson("granite", eos.TILLOTSON["granite"])]


def table_materials(n=200):
    """material 0 = iron, 1 = dunite, 2 = granite (synthetic rho-u tables)."""
    return [eos.synthetic_table(m, n, n) for m in ("iron", "dunite", "granite")]


MODE2_TABLES = ("iron120", "fine", "dunite200")


def mode2_table(g, name):
    """a table of the eos_mode2.npz fixture: regenerated from its synthetic_table spec, or stored"""
    import ast
    spec = ast.literal_eval(str(g[f"{name}_spec"]))
    if spec is not None:
        return eos.synthetic_table(**spec)
    a = {f: g[f"{name}_table_{f}"] for f in ("rho", "u", "pres", "snds", "temp", "ent")}
    return eos.Table(name=name, **a)


def mode2_materials():
    """material 0 = iron, 1 = dunite: 120 x 120 synthetic tables that reach down to 1e-3 kg/m^3,
    so every density above the floor (5) has a defined mode-2 lookup"""
    return [eos.synthetic_table(m, 120, 120, rho_range=(1e-3, 3e4)) for m in ("iron", "dunite")]


def oracle_config(materials, **kw):
    from oracle import pyoracle as po
    ms = po.MaterialSet([m.as_material() for m in materials])
    return po.make_config(ms, **kw)


def device_context(materials, **kw):
    from fdps_sph_gb300 import lib
    ctx = lib.Context(**kw)
    for k, m in enumerate(materials):
        ctx.set_material(k, m)
    return ctx


def small_impact(n_target=1800, n_impactor=200, seed=11, stir=True):
    """Two-body impact; with ``stir`` each body also spins and carries a
    seeded velocity noise, so div v, curl v, AV and du/dt are non-zero."""
    F, ids, mats, info = ic.config_small_impact(seed=seed, n_target=n_target, n_impactor=n_impactor)
    if stir:
        rng = np.random.default_rng(seed + 1000)
        X = F[[0, 1, 2]].T
        V = 1.0e-4 * np.cross(np.array([0.3, -0.2, 1.0]), X) + rng.normal(scale=30.0, size=X.shape)
        F[[3, 4, 5]] += V.T
    return F, ids, mats, info


def by_id(F, ids):
    o = np.argsort(ids, kind="stable")
    return F[:, o]


def rel_err(a, b, floor):
    floor = max(float(floor), 1e-300)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))) if len(a) else 0.0


def vec_rel_err(A, B, floor_frac=1e-6):
    """max_i |A_i - B_i| / max(|B_i|, floor_frac * max_k |B_k|) for rows of 3-vectors."""
    nb = np.linalg.norm(B, axis=1)
    fl = max(floor_frac * (nb.max() if len(nb) else 1.0), 1e-300)
    return float(np.max(np.linalg.norm(A - B, axis=1) / np.maximum(nb, fl))) if len(nb) else 0.0


def vec_err_rms(A, B):
    """max_i |A_i - B_i| / max(|B_i|, rms_k |B_k|): relative error of each
    particle's vector, floored at the RMS magnitude over all particles so
    that vectors which nearly cancel (interior of a uniform layer) are not
    judged by their own, arbitrarily small, magnitude."""
    nb = np.linalg.norm(B, axis=1)
    rms = float(np.sqrt(np.mean(nb * nb))) if len(nb) else 1.0
    return float(np.max(np.linalg.norm(A - B, axis=1) / np.maximum(nb, max(rms, 1e-300)))) if len(nb) else 0.0


def scalar_err_rms(a, b):
    rms = float(np.sqrt(np.mean(b * b))) if len(b) else 1.0
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), max(rms, 1e-300)))) if len(b) else 0.0
