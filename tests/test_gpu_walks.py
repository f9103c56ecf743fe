"""The MultiWalk loop over the functor-compatible batch entry points (fdps_sph_gb300.walks).

Walks of every gravity group of a 20,000-particle impact are run through sph_dispatch_* /
sph_retrieve_* the way calcForceAllAndWriteBackMultiWalk drives them (batches of n_walk_limit
walks over several tags).  The gravity walks carry the device's own EPJ / SPJ lists, so their
result is the FP64 context's gravity up to the summation order; the SPH walks carry FDPS-style
group supersets, on which the derivative and the hydro acceleration and du/dt equal the exact
sets' (W and grad W vanish beyond the support; only the hydro dt sees the superset)."""
import numpy as np
import pytest

from fdps_sph_gb300 import lib, walks
from fdps_sph_gb300.ic import FIELD
from helpers import device_context, scalar_err_rms, small_impact, tillotson_materials, vec_err_rms

pytestmark = pytest.mark.gpu


def test_multiwalk_matches_the_device_resident_forces():
    F, ids, mats, _ = small_impact(18000, 2000, seed=41)
    ctx = device_context(tillotson_materials(), precision=lib.PREC_FP64)
    try:
        ctx.upload(F, ids, mats)
        ctx.prologue()
        W = walks.Walks(ctx)
    finally:
        ctx.close()
    S = W.sorted_state
    assert W.n == F.shape[1] and int(W.count.sum()) == W.n
    for kind in ("drvt", "hydro", "grav"):
        W.run(kind, n_walk_limit=16, n_tags=3)
    g = W.result["grav"]
    assert vec_err_rms(g["acc"], np.stack([S[FIELD[c]] for c in ("gx", "gy", "gz")], 1)) < 1e-12
    assert scalar_err_rms(g["pot"], S[FIELD["pot"]]) < 1e-12
    hres = W.result["hydro"]
    assert vec_err_rms(hres["acc"], np.stack([S[FIELD[c]] for c in ("ax", "ay", "az")], 1)) < 1e-10
    assert scalar_err_rms(hres["eng_dot"], S[FIELD["eng_dot"]]) < 1e-10
    d = W.result["drvt"]
    assert scalar_err_rms(d["div_v"], S[FIELD["div_v"]]) < 1e-10
    assert np.max(np.abs(d["grad_smth"] - S[FIELD["grad_smth"]])) < 1e-12
    # the density walks run too (their result is the next density pass of the state's h)
    W.run("dens", n_walk_limit=16, n_tags=3)
    assert np.all(W.result["dens"]["dens"] > 0)


def test_multiwalk_mixed_precision_within_bar():
    """the same walks with sph_batch_set_precision(SPH_PREC_MIXED): gravity, hydro acceleration and
    du/dt and div v within 1e-5 of the FP64 context (floored at the RMS)"""
    F, ids, mats, _ = small_impact(18000, 2000, seed=42)
    ctx = device_context(tillotson_materials(), precision=lib.PREC_FP64)
    try:
        ctx.upload(F, ids, mats)
        ctx.prologue()
        W = walks.Walks(ctx)
    finally:
        ctx.close()
    S = W.sorted_state
    lib.batch_precision("mixed")
    try:
        for kind in ("drvt", "hydro", "grav"):
            W.run(kind, n_walk_limit=64, n_tags=2)
    finally:
        lib.batch_precision("fp64")
    g, hres, d = W.result["grav"], W.result["hydro"], W.result["drvt"]
    assert vec_err_rms(g["acc"], np.stack([S[FIELD[c]] for c in ("gx", "gy", "gz")], 1)) < 1e-5
    assert scalar_err_rms(g["pot"], S[FIELD["pot"]]) < 1e-5
    assert vec_err_rms(hres["acc"], np.stack([S[FIELD[c]] for c in ("ax", "ay", "az")], 1)) < 1e-5
    assert scalar_err_rms(hres["eng_dot"], S[FIELD["eng_dot"]]) < 1e-5
    assert scalar_err_rms(d["div_v"], S[FIELD["div_v"]]) < 1e-5


def test_multiwalk_index_form_equals_payload_form():
    """the same walks through the index form (each pass's EPJ / SPJ arrays sent once, the walks as
    indices): bit-identical to the payload form in FP64 and in mixed precision"""
    F, ids, mats, _ = small_impact(18000, 2000, seed=43)
    ctx = device_context(tillotson_materials(), precision=lib.PREC_FP64)
    try:
        ctx.upload(F, ids, mats)
        ctx.prologue()
        W = walks.Walks(ctx)
    finally:
        ctx.close()
    for precision in ("fp64", "mixed"):
        lib.batch_precision(precision)
        try:
            for kind in walks.KINDS:
                W.run(kind, n_walk_limit=64, n_tags=3)
                ref = W.result[kind].copy()
                W.run(kind, n_walk_limit=64, n_tags=3, index=True)
                assert W.result[kind].tobytes() == ref.tobytes(), (precision, kind)
        finally:
            lib.batch_precision("fp64")
