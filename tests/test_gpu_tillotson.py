"""The device's analytic Tillotson EoS against the reference's own branches.

tillotson.npz holds P_co and P_ex of the reference's Tillotson class (EoS.h:91-103) with the
granite (EoS.h:446) and iron (EoS.h:448) parameters.  The device evaluates the same operations
in the same order, so each pure branch agrees to a few ulps (nvcc may fuse a multiply and an add
the reference rounds twice, so the bar is 1e-13 of the largest term of the branch); the blend
region (this project's regime rule, linear in u between uiv and ucv) is checked against the same
rule applied to the reference's two values."""
import numpy as np
import pytest

from fdps_sph_gb300 import eos, lib
from helpers import load_golden

pytestmark = pytest.mark.gpu

TIL_COMPRESSED, TIL_COLD, TIL_HOT, TIL_BLEND = 0, 1, 2, 3


def _term_scale(par, rho, u):
    """the largest magnitude among the terms of P_co and P_ex at (rho, u): the size of the
    rounding a sum of them can carry"""
    rho0, u0, _, _, A, B, a, b, alpha, beta = par
    eta = rho / rho0
    mu = eta - 1.0
    om = u / u0 / eta / eta + 1.0
    z = 1.0 / eta - 1.0
    terms = [a * rho * u, b * rho * u / om, A * np.abs(mu), B * mu * mu, A * np.abs(mu) * np.exp(-alpha * z)]
    return np.max(np.abs(np.stack(terms)), axis=0)


@pytest.mark.parametrize("name", ["granite", "iron"])
def test_device_tillotson_matches_reference_branches(name):
    g = load_golden("tillotson.npz")
    par = g[f"{name}_par"]
    rho, u, reg = g[f"{name}_rho"], g[f"{name}_u"], g[f"{name}_region"]
    pco, pex = g[f"{name}_P_co"], g[f"{name}_P_ex"]
    uiv, ucv = par[2], par[3]
    want = np.where((reg == TIL_COMPRESSED) | (reg == TIL_COLD), pco,
                    np.where(reg == TIL_HOT, pex, ((u - uiv) * pex + (ucv - u) * pco) / (ucv - uiv)))
    ctx = lib.Context()
    try:
        ctx.set_material(0, eos.Tillotson(name, tuple(par)))
        P, _ = ctx.eos_eval(0, "pressure", rho, u)
        cs, _ = ctx.eos_eval(0, "sound_speed", rho, u)
    finally:
        ctx.close()
    err = np.abs(P - want) / _term_scale(par, rho, u)
    assert np.max(err) < 1e-13, (name, float(np.max(err)), int(np.argmax(err)))
    assert np.all(np.isfinite(cs)) and np.all(cs > 0)
