"""Error of the mixed-precision path against the plain FP64 path on one state.

Both paths evaluate the forces of the same particle state: the state is
uploaded into a fresh context of each precision and its prologue is run
(main.cpp:92-105: four density passes, EoS, derivative, hydro force and
gravity of the current positions and velocities).  The FP64 path is the one
the parity tests hold to the CPU oracle at 1e-10, so these numbers are the
mixed path's error against the oracle's arithmetic.

Error measures, per particle, maximum over particles:
  * density and potential: relative, |a - b| / |b|;
  * hydro acceleration, gravity, their sum and du/dt: |a - b| / max(|b|,
    rms_k |b_k|), the RMS over all particles flooring the denominator so
    that quantities which nearly cancel (a particle at rest in a uniform
    layer) are not judged by their own, arbitrarily small, magnitude.
"""
from __future__ import annotations

import numpy as np

from .ic import FIELD

ERR_FIELDS = ("dens", "ax", "ay", "az", "eng_dot", "gx", "gy", "gz", "pot", "div_v")


def _vec(F, keys):
    return np.stack([F[FIELD[k]] for k in keys], 1)


def vec_err_each(A, B):
    """per particle |A_i - B_i| / max(|B_i|, rms_k |B_k|)"""
    nb = np.linalg.norm(B, axis=1)
    rms = max(float(np.sqrt(np.mean(nb * nb))), 1e-300)
    return np.linalg.norm(A - B, axis=1) / np.maximum(nb, rms)


def scalar_err_each(a, b, floor_rms=True):
    """per particle |a_i - b_i| / max(|b_i|, rms_k |b_k|) (floor_rms) or / |b_i|"""
    rms = max(float(np.sqrt(np.mean(b * b))), 1e-300) if floor_rms else 1e-300
    return np.abs(a - b) / np.maximum(np.abs(b), rms)


def vec_err_rms(A, B):
    return float(np.max(vec_err_each(A, B)))


def scalar_err_rms(a, b):
    return float(np.max(scalar_err_each(a, b)))


def _quantities(Fm, Ff):
    acc = ("ax", "ay", "az")
    grav = ("gx", "gy", "gz")
    return {
        "dens": (Fm[FIELD["dens"]], Ff[FIELD["dens"]], False),
        "acc_hydro": (_vec(Fm, acc), _vec(Ff, acc), True),
        "eng_dot": (Fm[FIELD["eng_dot"]], Ff[FIELD["eng_dot"]], True),
        "acc_grav": (_vec(Fm, grav), _vec(Ff, grav), True),
        "pot": (Fm[FIELD["pot"]], Ff[FIELD["pot"]], False),
        "acc_total": (_vec(Fm, acc) + _vec(Fm, grav), _vec(Ff, acc) + _vec(Ff, grav), True),
    }


def _each(a, b, floored):
    return vec_err_each(a, b) if a.ndim == 2 else scalar_err_each(a, b, floored)


def force_errors(Fm, Ff):
    """per-quantity error of the field block Fm (mixed) against Ff (FP64), both in id order: the
    maximum over particles (density and potential relative per particle; vectors and du/dt floored
    at the RMS over particles)"""
    return {k: float(np.max(_each(a, b, fl))) for k, (a, b, fl) in _quantities(Fm, Ff).items()}


def error_distribution(Fm, Ff):
    """the per-particle errors of force_errors as quantiles (p50, p99, p99.9, max), and the global
    relative L2 error ||a - b|| / ||b|| over all particles, per quantity"""
    out = {}
    for k, (a, b, fl) in _quantities(Fm, Ff).items():
        e = _each(a, b, fl)
        q = np.quantile(e, [0.5, 0.99, 0.999])
        out[k] = {"p50": float(q[0]), "p99": float(q[1]), "p99.9": float(q[2]), "max": float(np.max(e)),
                  "l2_rel": float(np.linalg.norm(a - b) / max(float(np.linalg.norm(b)), 1e-300))}
    return out


def activity(F):
    """how active the hydro is in a state whose forces are in F: the fraction of particles under
    compression (div v < 0: their approaching neighbours enter the artificial viscosity,
    force.h:124-131) and the RMS and maximum |du/dt| (zero while bodies move rigidly)"""
    divv = F[FIELD["div_v"]]
    ed = F[FIELD["eng_dot"]]
    return {"frac_compressing": float(np.mean(divv < 0.0)),
            "eng_dot_rms": float(np.sqrt(np.mean(ed * ed))),
            "eng_dot_max_abs": float(np.max(np.abs(ed)))}


def by_id(F, ids):
    return F[:, np.argsort(ids, kind="stable")]


def forces_of_state(F, ids, mats, materials, precision, theta=0.5, device=0, time=0.0):
    """the prologue forces of state F (field-major, any order) in a fresh context; returned in
    id order, with the context's per-segment timings switched off"""
    from . import lib
    ctx = lib.Context(precision=precision, device=device, theta=theta)
    try:
        for k, m in enumerate(materials):
            ctx.set_material(k, m)
        ctx.upload(F, ids, mats, time=time)
        ctx.prologue()
        Fo, io, _ = ctx.download()
    finally:
        ctx.close()
    return by_id(Fo, io)


def compare_on_state(F, ids, mats, materials, theta=0.5, device=0, time=0.0):
    """errors of the mixed path's forces against the FP64 path's on state F, and the state's
    activity measured by the FP64 forces"""
    Fm = forces_of_state(F, ids, mats, materials, "mixed", theta, device, time)
    Ff = forces_of_state(F, ids, mats, materials, "fp64", theta, device, time)
    out = force_errors(Fm, Ff)
    out["activity"] = activity(Ff)
    out["distribution"] = error_distribution(Fm, Ff)
    return out


def passes_of_state(F, ids, mats, materials, precision, theta=0.5, device=0, time=0.0):
    """the derivative and hydro forces of state F evaluated pass by pass (sph_run_pass: sort and
    octree, EoS, derivative, hydro) on the density and smoothing length F carries, instead of a
    prologue's own density passes; returned in id order"""
    from . import lib
    ctx = lib.Context(precision=precision, device=device, theta=theta)
    try:
        for k, m in enumerate(materials):
            ctx.set_material(k, m)
        ctx.upload(F, ids, mats, time=time)
        for p in (0, 2, 3, 4):
            ctx.run_pass(p)
        Fo, io, _ = ctx.download()
    finally:
        ctx.close()
    return by_id(Fo, io)


def hydro_error_sources(F, ids, mats, materials, theta=0.5, device=0, time=0.0):
    """where the mixed path's hydro error on state F comes from: the error of a_hydro and du/dt
    against the FP64 prologue (p99.9 and max, measures of force_errors) for
      mixed            -- the mixed prologue (density and pairs in mixed precision);
      mixed_pairs      -- mixed derivative and hydro on the FP64 prologue's density and h;
      mixed_density    -- FP64 derivative and hydro on the mixed prologue's density and h;
      fp64_passes      -- FP64 derivative and hydro on the FP64 density and h (zero: the pass
                          sequence reproduces the prologue)"""
    Ff = forces_of_state(F, ids, mats, materials, "fp64", theta, device, time)
    Fm = forces_of_state(F, ids, mats, materials, "mixed", theta, device, time)
    order = np.argsort(ids, kind="stable")
    S, sid, smat = F[:, order], ids[order], mats[order]

    def with_dens(src):
        X = S.copy()
        for k in ("dens", "smth"):
            X[FIELD[k]] = src[FIELD[k]]
        return X

    runs = {"mixed": Fm,
            "mixed_pairs": passes_of_state(with_dens(Ff), sid, smat, materials, "mixed", theta, device, time),
            "mixed_density": passes_of_state(with_dens(Fm), sid, smat, materials, "fp64", theta, device, time),
            "fp64_passes": passes_of_state(with_dens(Ff), sid, smat, materials, "fp64", theta, device, time)}
    out = {}
    for name, X in runs.items():
        q = _quantities(X, Ff)
        out[name] = {}
        for k in ("acc_hydro", "eng_dot"):
            a, b, fl = q[k]
            e = _each(a, b, fl)
            out[name][k] = {"p99.9": float(np.quantile(e, 0.999)), "max": float(np.max(e))}
    return out
