"""Mode 2 (main.cpp:155-158: SetConstantEntropy + CalcAll, force.h:55-84) on the
device, through the C ABI, against the oracle and the reference's own outputs.

* sph_eos_eval: InternalEnergy (RestrictedBilinearInterpolation,
  interpolation.h:107-335), Temperature, Entropy, Pressure and SoundSpeed at
  the golden points of tests/golden/eos_mode2.npz, for both resolutions of the
  reference's abs(); energies bit-identical to the oracle and the reference.
* sph_step in mode 2 against or_step (FP64), mixed against FP64, the batched
  path (a run alone equals the run in a mix), and the failure of a step whose
  lookups are undefined in the reference.
"""
import numpy as np
import pytest

from helpers import (MODE2_TABLES, by_id, device_context, load_golden, mode2_materials, mode2_table, oracle_config,
                     rel_err, small_impact, vec_err_rms)

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", MODE2_TABLES)
@pytest.mark.parametrize("abs_mode", [0, 1])
def test_internal_energy_matches_reference(name, abs_mode):
    from oracle import pyoracle as po
    g = load_golden("eos_mode2.npz")
    t = mode2_table(g, name)
    ctx = device_context([t], entropy_abs=abs_mode)
    pts = g[f"{name}_points"]
    U, undef = ctx.eos_eval(0, "internal_energy", pts[:, 0], pts[:, 1])
    ref = g[f"{name}_U_int" if abs_mode == 0 else f"{name}_U_real"]
    assert undef == 0
    assert np.array_equal(U, ref)     # FP64 in the reference's operation order: bit-identical
    # points where the reference's lookup is NaN or undefined: same as the oracle
    ms = po.MaterialSet([t.as_material()])
    e = g[f"{name}_edges"]
    Ue, undef_e = ctx.eos_eval(0, "internal_energy", e[:, 0], e[:, 1])
    orc = [ms.internal_energy(0, r, s, 120, abs_mode) for r, s, _ in e]
    assert undef_e == sum(u for _, u in orc)
    ov = np.array([v for v, _ in orc])
    assert np.array_equal(np.isnan(Ue), np.isnan(ov))
    assert np.array_equal(Ue[~np.isnan(ov)], ov[~np.isnan(ov)])
    ctx.close()


@pytest.mark.parametrize("name", MODE2_TABLES)
def test_temperature_entropy_pressure_match(name):
    from oracle import pyoracle as po
    g = load_golden("eos_mode2.npz")
    t = mode2_table(g, name)
    ctx = device_context([t])
    pts = g[f"{name}_points"]
    T, _ = ctx.eos_eval(0, "temperature", pts[:, 0], pts[:, 2])
    S, _ = ctx.eos_eval(0, "entropy", pts[:, 0], pts[:, 2])
    assert rel_err(T, g[f"{name}_T"], 1e-300) < 1e-13
    assert rel_err(S, g[f"{name}_S"], 1e-9 * np.abs(g[f"{name}_S"]).max()) < 1e-12
    ms = po.MaterialSet([t.as_material()])
    P, _ = ctx.eos_eval(0, "pressure", pts[:, 0], pts[:, 2])
    C, _ = ctx.eos_eval(0, "sound_speed", pts[:, 0], pts[:, 2])
    o = np.array([ms.eval(0, r, u) for r, _, u in pts])
    assert rel_err(P, o[:, 0], 1e-9 * np.abs(o[:, 0]).max()) < 1e-12
    assert rel_err(C, o[:, 1], 1e-300) < 1e-12
    ctx.close()


def test_ideal_gas_surface():
    """IdealGas (EoS.h:37-66): P and c_s analytic, InternalEnergy / Temperature / Entropy 0"""
    from fdps_sph_gb300 import eos
    ctx = device_context([eos.IdealGas(5.0 / 3.0)])
    rho = np.array([1.0, 10.0, 3.0e3])
    u = np.array([1.0e5, 2.0e6, 7.0e3])
    P, _ = ctx.eos_eval(0, "pressure", rho, u)
    C, _ = ctx.eos_eval(0, "sound_speed", rho, u)
    assert rel_err(P, (2.0 / 3.0) * rho * u, 1e-300) < 1e-15
    assert rel_err(C, np.sqrt((5.0 / 3.0) * (2.0 / 3.0) * u), 1e-300) < 1e-15
    for q in ("internal_energy", "temperature", "entropy"):
        v, und = ctx.eos_eval(0, q, rho, u)
        assert und == 0 and np.all(v == 0.0)
    ctx.close()


def _mode2_case(n_target=1800, n_impactor=200, seed=11):
    F, ids, mats, _ = small_impact(n_target, n_impactor, seed)
    return F, ids, mats


M2 = dict(mode=2, mantle_entropy=3100.0, core_entropy=2500.0)


def test_mode2_steps_match_oracle():
    """FP64 device steps in mode 2 against or_step: the energy and temperature written by
    CalcAll, and the trajectory they feed, within the FP64 parity bound"""
    from oracle import pyoracle as po
    from fdps_sph_gb300.ic import FIELD
    F, ids, mats = _mode2_case()
    mat = mode2_materials()
    s = po.OracleSystem(F, ids, mats)
    s.initialize_smth()
    cfg = oracle_config(mat, **M2)
    s.prologue(cfg)
    s.step(cfg, 4)
    ctx = device_context(mat, precision=0, **M2)
    ctx.upload(F, ids, mats, init_smth=True)
    ctx.prologue()
    ctx.step(4)
    Fd, idd, _ = ctx.download()
    ctx.close()
    Fo, ido, _ = s.by_id()
    Fd = by_id(Fd, idd)
    assert np.array_equal(np.sort(idd), ido)
    assert np.array_equal(Fd[FIELD["ent"]], Fo[FIELD["ent"]])
    assert set(np.unique(Fd[FIELD["ent"]])) == {3100.0, 2500.0}
    for f in ("dens", "eng", "temp", "pot"):
        assert rel_err(Fd[FIELD[f]], Fo[FIELD[f]], 1e-300) < 1e-10, f
    for v in (("x", "y", "z"), ("vx", "vy", "vz"), ("ax", "ay", "az"), ("gx", "gy", "gz")):
        A = np.stack([Fd[FIELD[c]] for c in v], 1)
        B = np.stack([Fo[FIELD[c]] for c in v], 1)
        assert vec_err_rms(A, B) < 1e-10, v


def test_mode2_mixed_matches_fp64():
    from fdps_sph_gb300.ic import FIELD
    F, ids, mats = _mode2_case(9000, 1000, 5)
    mat = mode2_materials()
    out = {}
    for prec in (0, 1):
        ctx = device_context(mat, precision=prec, **M2)
        ctx.upload(F, ids, mats, init_smth=True)
        ctx.prologue()
        ctx.step(3)
        Fd, idd, _ = ctx.download()
        out[prec] = by_id(Fd, idd)
        ctx.close()
    for f in ("dens", "eng", "temp"):
        a, b = out[1][FIELD[f]], out[0][FIELD[f]]
        assert rel_err(a, b, 1e-300) < 1e-5, f


@pytest.mark.parametrize("prec", [0, 1])
def test_mode2_run_in_a_mix_equals_run_alone(prec):
    """a run added to a context in mode 2 takes its first step as its prologue (no CalcAll,
    as before the reference's loop) and then matches the run advanced alone bit for bit"""
    a = _mode2_case(1500, 150, 21)
    b = _mode2_case(700, 120, 22)
    mat = mode2_materials()
    ctx = device_context(mat, precision=prec, **M2)
    ha = ctx.add_run(*a)
    ctx.step(1 + 2)
    hb = ctx.add_run(*b)
    ctx.step(1 + 3)
    for h, body, steps in ((ha, a, 6), (hb, b, 3)):
        alone = device_context(mat, precision=prec, **M2)
        alone.upload(*body)
        alone.prologue()
        alone.step(steps)
        x, y = ctx.download_run(h), alone.download()
        alone.close()
        assert np.array_equal(x[1], y[1])
        assert np.array_equal(x[0], y[0]), float(np.nanmax(np.abs(x[0] - y[0])))
    ctx.close()


def test_mode2_undefined_lookup_fails_the_step():
    """200-column tables with the reference's 120-line slices: the lookups index outside the
    reference's vectors, and the step reports it instead of carrying NaN energies"""
    from fdps_sph_gb300 import eos, lib
    F, ids, mats = _mode2_case(900, 100, 3)
    mat = [eos.synthetic_table(m, 200, 200) for m in ("iron", "dunite")]
    ctx = device_context(mat, precision=1, **M2)
    ctx.upload(F, ids, mats, init_smth=True)
    ctx.prologue()
    with pytest.raises(lib.SphError) as ei:
        ctx.step(1)
    assert ei.value.code == -5 and "mode 2" in str(ei.value)
    ctx.close()
