"""Mixed precision against FP64 on a colliding state.

The prologue forces of two bodies far apart are a weak test of the hydro
force: every particle moves rigidly, so no pair approaches (the artificial
viscosity of force.h:124-131 is off) and du/dt is zero in both paths.  Here a
100,000-particle impact starts with the bodies in contact and takes ten
mixed-precision steps, so the contact region is shocked; that state's forces
are then evaluated by both paths and held to the 1e-5 bar (density and
potential relative per particle; vectors and du/dt relative per particle,
floored at the RMS over particles).  The FP64 path is the one the parity
tests hold to the oracle."""
import numpy as np
import pytest

from fdps_sph_gb300 import accuracy, eos, ic, lib

pytestmark = pytest.mark.gpu


def test_mixed_against_fp64_on_a_shocked_contact_state():
    F, ids, mats, _ = ic.config_1m_contact(seed=31, n_target=90_000, n_impactor=10_000)
    materials = [eos.synthetic_table(m) for m in ("iron", "dunite")]
    ctx = lib.Context(precision="mixed")
    try:
        for k, m in enumerate(materials):
            ctx.set_material(k, m)
        ctx.upload(F, ids, mats)
        ctx.prologue()
        ctx.step(10)
        t, _, _ = ctx.time()
        S, sid, smat = ctx.download()
    finally:
        ctx.close()
    errs = accuracy.compare_on_state(S, sid, smat, materials, time=t)
    act = errs.pop("activity")
    dist = errs.pop("distribution")
    print("mixed vs FP64 on the shocked contact state:", errs, act, dist)
    # the state is active: particles under compression and non-zero du/dt
    assert act["frac_compressing"] > 0.01 and act["eng_dot_rms"] > 0.0
    for k, v in errs.items():
        assert v < 1e-5, (k, v)


def test_hydro_error_sources_on_a_shocked_contact_state():
    """the mixed hydro error split between the density (through the pressure) and the pair
    arithmetic: re-evaluating the derivative and hydro passes on the other path's density.  The
    FP64 passes on the FP64 density reproduce the FP64 prologue exactly, and each source alone
    stays within the bar"""
    F, ids, mats, _ = ic.config_1m_contact(seed=32, n_target=90_000, n_impactor=10_000)
    materials = [eos.synthetic_table(m) for m in ("iron", "dunite")]
    ctx = lib.Context(precision="mixed")
    try:
        for k, m in enumerate(materials):
            ctx.set_material(k, m)
        ctx.upload(F, ids, mats)
        ctx.prologue()
        ctx.step(10)
        t, _, _ = ctx.time()
        S, sid, smat = ctx.download()
    finally:
        ctx.close()
    src = accuracy.hydro_error_sources(S, sid, smat, materials, time=t)
    print("hydro error sources:", src)
    assert src["fp64_passes"]["acc_hydro"]["max"] == 0.0 and src["fp64_passes"]["eng_dot"]["max"] == 0.0
    for name in ("mixed", "mixed_pairs", "mixed_density"):
        for k in ("acc_hydro", "eng_dot"):
            assert src[name][k]["max"] < 1e-5, (name, k)
