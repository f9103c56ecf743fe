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


def vec_err_rms(A, B):
    nb = np.linalg.norm(B, axis=1)
    rms = max(float(np.sqrt(np.mean(nb * nb))), 1e-300)
    return float(np.max(np.linalg.norm(A - B, axis=1) / np.maximum(nb, rms)))


def scalar_err_rms(a, b):
    rms = max(float(np.sqrt(np.mean(b * b))), 1e-300)
    return float(np.max(np.abs(a - b) / np.maximum(np.abs(b), rms)))


def force_errors(Fm, Ff):
    """per-quantity error of the field block Fm (mixed) against Ff (FP64), both in id order"""
    acc = ("ax", "ay", "az")
    grav = ("gx", "gy", "gz")
    return {
        "dens": float(np.max(np.abs(Fm[FIELD["dens"]] - Ff[FIELD["dens"]]) / np.abs(Ff[FIELD["dens"]]))),
        "acc_hydro": vec_err_rms(_vec(Fm, acc), _vec(Ff, acc)),
        "eng_dot": scalar_err_rms(Fm[FIELD["eng_dot"]], Ff[FIELD["eng_dot"]]),
        "acc_grav": vec_err_rms(_vec(Fm, grav), _vec(Ff, grav)),
        "pot": float(np.max(np.abs(Fm[FIELD["pot"]] - Ff[FIELD["pot"]]) / np.abs(Ff[FIELD["pot"]]))),
        "acc_total": vec_err_rms(_vec(Fm, acc) + _vec(Fm, grav), _vec(Ff, acc) + _vec(Ff, grav)),
    }


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
    return out
