"""The CPU oracle (oracle/sph_oracle.c) against golden vectors produced by
the reference's own code (tests/golden/make_golden.py)."""
import ast
import os

import numpy as np
import pytest

from fdps_sph_gb300 import eos, ic
from oracle import pyoracle as po

GOLD = os.path.join(os.path.dirname(__file__), "golden")


def load(name):
    return np.load(os.path.join(GOLD, name), allow_pickle=False)


def relerr(a, b, floor):
    return np.max(np.abs(a - b) / np.maximum(np.abs(b), floor))


def test_kernel_matches_reference():
    g = load("kernel.npz")
    W = np.array([po.kernel_W(*d, h) for d, h in zip(g["dr"], g["h"])])
    gW = np.array([po.kernel_gradW(*d, h) for d, h in zip(g["dr"], g["h"])])
    assert relerr(W, g["W"], 1e-300) < 1e-13
    scale = np.abs(g["gradW"]).max(axis=1, keepdims=True) + 1e-300
    assert np.max(np.abs(gW - g["gradW"]) / scale) < 1e-13
    # the self term has zero gradient, not NaN
    assert np.all(gW[:8] == 0.0)


@pytest.mark.parametrize("fixture", ["eos_small.npz", "eos_dunite200.npz"])
def test_table_lookup_matches_reference(fixture):
    g = load(fixture)
    spec = ast.literal_eval(str(g["spec"]))
    t = eos.synthetic_table(spec["material"], spec["n_rho"], spec["n_u"], spec["rho_range"], spec["u_range"])
    # table regeneration is bit-identical to the one the reference read
    assert np.array_equal(t.rho, g["rho"]) and np.array_equal(t.u, g["u"])
    assert np.array_equal(t.pres, g["pres"]) and np.array_equal(t.snds, g["snds"])
    ms = po.MaterialSet([t.as_material()])
    out = np.array([ms.eval(0, r, u) for r, u in g["points"]])
    for col, ref in ((0, g["P"]), (1, g["cs"]), (0, g["P_til"]), (1, g["cs_til"])):
        floor = 1e-9 * np.abs(ref).max()
        assert relerr(out[:, col], ref, floor) < 1e-12


def _system(F, ids, mats):
    return po.OracleSystem(F, ids, mats)


def _materials():
    return po.MaterialSet([eos.Tillotson("iron", eos.TILLOTSON["iron"]).as_material(),
                           eos.Tillotson("granite", eos.TILLOTSON["granite"]).as_material()])


@pytest.fixture(scope="module")
def fun():
    return load("functors.npz")


def test_resort_is_identity(fun):
    s = _system(fun["state_dens"], fun["ids"], fun["mats"])
    po.OracleTree(s)
    assert np.array_equal(s.id, fun["ids"])


def test_density_matches_reference(fun):
    s = _system(fun["state_dens"], fun["ids"], fun["mats"])
    tr = po.OracleTree(s)
    tr.pass_density(po.make_config(_materials()))
    ref = fun["ref_dens"]
    assert relerr(s.field("dens"), ref["dens"], 1e-300) < 1e-12
    assert relerr(s.field("smth"), ref["smth"], 1e-300) < 1e-12


def test_derivative_and_balsara_match_reference(fun):
    s = _system(fun["state_drvt"], fun["ids"], fun["mats"])
    tr = po.OracleTree(s)
    tr.pass_derivative()
    ref = fun["ref_drvt"]
    dv = ref["div_v"]
    floor = 1e-9 * np.abs(dv).max()
    assert relerr(s.field("div_v"), dv, floor) < 1e-10
    rot = np.stack([s.field("rot_x"), s.field("rot_y"), s.field("rot_z")], axis=1)
    assert np.max(np.linalg.norm(rot - ref["rot_v"], axis=1) /
                  np.maximum(np.linalg.norm(ref["rot_v"], axis=1), 1e-9 * np.abs(ref["rot_v"]).max())) < 1e-10
    assert relerr(s.field("grad_smth"), ref["grad_smth"], 1e-300) < 1e-12
    assert relerr(s.field("bal"), fun["ref_bal"], 1e-12) < 1e-9


def test_hydro_matches_reference(fun):
    s = _system(fun["state_hydro"], fun["ids"], fun["mats"])
    tr = po.OracleTree(s)
    tr.pass_hydro()
    acc = np.stack([s.field("ax"), s.field("ay"), s.field("az")], axis=1)
    for key in ("ref_hydro_superset", "ref_hydro_exact"):
        ref = fun[key]
        an = np.linalg.norm(ref["acc"], axis=1)
        assert np.max(np.linalg.norm(acc - ref["acc"], axis=1) / np.maximum(an, 1e-6 * an.max())) < 1e-10
        ed = ref["eng_dot"]
        assert relerr(s.field("eng_dot"), ed, 1e-6 * np.abs(ed).max()) < 1e-10
    # dt: v_sig_max over the exact symmetric neighbour set
    assert relerr(s.field("dt"), fun["ref_hydro_exact"]["dt"], 1e-300) < 1e-13
    # the superset walk can only raise v_sig_max, i.e. lower dt
    assert np.all(fun["ref_hydro_superset"]["dt"] <= fun["ref_hydro_exact"]["dt"] * (1 + 1e-14))


def test_gravity_matches_reference(fun):
    s = _system(fun["state_hydro"], fun["ids"], fun["mats"])
    tr = po.OracleTree(s)
    tr.pass_gravity(po.make_config(_materials()))
    ref = fun["ref_grav"]
    g = np.stack([s.field("gx"), s.field("gy"), s.field("gz")], axis=1)
    gn = np.linalg.norm(ref["acc"], axis=1)
    assert np.max(np.linalg.norm(g - ref["acc"], axis=1) / np.maximum(gn, 1e-6 * gn.max())) < 1e-11
    assert relerr(s.field("pot"), ref["pot"], 1e-300) < 1e-12


def test_integrator_matches_reference():
    g = load("integ.npz")
    rec, out = g["rec"], g["out"]
    n = len(rec)
    F = np.zeros((po.NFIELD, n))
    for k, name in enumerate(["x", "y", "z", "vx", "vy", "vz", "ax", "ay", "az", "gx", "gy", "gz", "eng",
                              "eng_dot"]):
        F[po.FIELD[name]] = rec[:, k]
    s = po.OracleSystem(F, np.arange(n), np.zeros(n, np.int32))
    dt, damp = float(g["dt"]), float(g["damping"])
    po.kick_drift_predict(s, dt)
    got1 = np.stack([s.field(k) for k in ["x", "y", "z", "vx", "vy", "vz", "vhx", "vhy", "vhz", "eng",
                                          "eng_half"]], axis=1)
    assert np.max(np.abs(got1 - out[:, :11]) / np.maximum(np.abs(out[:, :11]), 1e-300)) < 1e-14
    for k, name in enumerate(["ax", "ay", "az", "gx", "gy", "gz", "eng_dot"]):
        s.F[po.FIELD[name]] = rec[:, 14 + k]
    po.final_kick(s, dt, damp)
    got2 = np.stack([s.field(k) for k in ["vx", "vy", "vz", "eng"]], axis=1)
    assert np.max(np.abs(got2 - out[:, 11:]) / np.maximum(np.abs(out[:, 11:]), 1e-300)) < 1e-14


def test_dt_global_matches_reference():
    g = load("dtglobal.npz")
    rec = g["rec"]
    n = len(rec)
    F = np.zeros((po.NFIELD, n))
    F[po.FIELD["dt"]] = rec[:, 0]
    s = po.OracleSystem(F, np.arange(n), np.zeros(n, np.int32))
    assert po.dt_global(s) == float(g["dt"])


# --- mode 2: SetConstantEntropy + CalcAll (main.cpp:155-158) ------------------
@pytest.mark.parametrize("name", ["iron120", "fine", "dunite200"])
def test_mode2_eos_matches_reference(name):
    """InternalEnergy (RestrictedBilinearInterpolation), Temperature and Entropy of the
    oracle against the reference's ANEOS class, for both resolutions of abs()"""
    from helpers import mode2_table
    g = load("eos_mode2.npz")
    t = mode2_table(g, name)
    ms = po.MaterialSet([t.as_material()])
    pts = g[f"{name}_points"]
    assert len(pts) > 150
    for abs_mode, key in ((0, "U_int"), (1, "U_real")):
        got = np.array([ms.internal_energy(0, r, s, 120, abs_mode) for r, s, _ in pts])
        assert not got[:, 1].any()
        assert relerr(got[:, 0], g[f"{name}_{key}"], 1e-300) <= 1e-15
    T = np.array([ms.temperature(0, r, u) for r, _, u in pts])
    S = np.array([ms.entropy(0, r, u) for r, _, u in pts])
    assert relerr(T, g[f"{name}_T"], 1e-300) < 1e-13
    assert relerr(S, g[f"{name}_S"], 1e-9 * np.abs(g[f"{name}_S"]).max()) < 1e-12
    if name == "fine":   # the two abs() resolutions really differ on this table
        assert np.sum(g["fine_U_int"] != g["fine_U_real"]) > 100


def test_mode2_edges_are_flagged():
    """densities on a table row give NaN (0/0 in the density interpolation), densities above
    the table and entropies outside a slice index outside the reference's vectors"""
    from helpers import mode2_table
    g = load("eos_mode2.npz")
    t = mode2_table(g, "iron120")
    ms = po.MaterialSet([t.as_material()])
    e = g["iron120_edges"]
    res = [ms.internal_energy(0, r, s, 120, 0) for r, s, _ in e]
    vals = np.array([v for v, _ in res])
    und = np.array([u for _, u in res])
    assert np.all(np.isnan(vals[:8])) and not und[:8].any()    # rows: defined, NaN
    assert np.isnan(vals[8]) and not und[8]                      # below the table: p1 == p2
    assert und[9] and und[10]                                    # at / above the last row
    assert und[13] and np.isnan(vals[14])                        # |s - e| >= 2^31; NaN density
    # the 200-column table with the reference's 120-line slices: many undefined lookups
    t2 = mode2_table(g, "dunite200")
    ms2 = po.MaterialSet([t2.as_material()])
    rng = np.random.default_rng(1)
    r = np.exp(rng.uniform(np.log(t2.rho[1]), np.log(t2.rho[-2]), 200))
    und2 = [ms2.internal_energy(0, x, 3000.0, 120, 0)[1] for x in r]
    assert 0 < sum(und2) < 200


def test_mode2_step_sets_entropy_energy_temperature():
    """or_step in mode 2 ends with ent = mantle / core entropy by material and eng, temp from
    the tables at the step's density"""
    from helpers import mode2_materials, oracle_config, small_impact
    F, ids, mats, _ = small_impact(900, 100)
    mat = mode2_materials()
    cfg = oracle_config(mat, mode=2, mantle_entropy=3100.0, core_entropy=2500.0)
    s = po.OracleSystem(F, ids, mats)
    s.initialize_smth()
    s.prologue(cfg)
    s.step(cfg, 1)
    ms = po.MaterialSet([m.as_material() for m in mat])
    ent = s.field("ent")
    assert np.all(ent[s.mat == 0] == 3100.0) and np.all(ent[s.mat == 1] == 2500.0)
    for i in range(0, s.n, 97):
        u, und = ms.internal_energy(s.mat[i], s.field("dens")[i], ent[i])
        assert not und and u == s.field("eng")[i]
        assert ms.temperature(s.mat[i], s.field("dens")[i], u) == s.field("temp")[i]


TIL_COMPRESSED, TIL_COLD, TIL_HOT, TIL_BLEND = 0, 1, 2, 3


def tillotson_expected(g, name):
    """the pressure the regime rule picks from the reference's own branches (tillotson.npz):
    P_co where compressed or cold, P_ex where hot, linear in u between them in the blend region"""
    par = g[f"{name}_par"]
    uiv, ucv = par[2], par[3]
    reg, u = g[f"{name}_region"], g[f"{name}_u"]
    pco, pex = g[f"{name}_P_co"], g[f"{name}_P_ex"]
    blend = ((u - uiv) * pex + (ucv - u) * pco) / (ucv - uiv)
    return np.where((reg == TIL_COMPRESSED) | (reg == TIL_COLD), pco, np.where(reg == TIL_HOT, pex, blend))


def test_oracle_tillotson_branches_match_reference():
    """or_tillotson's pressure against the reference's P_co / P_ex (EoS.h:91-103): 1e-14 relative
    on every pure branch (same operations in the same order), the blend from the same two values
    to 1e-13 of the larger branch."""
    from fdps_sph_gb300 import eos
    g = load("tillotson.npz")
    for name in ("granite", "iron"):
        ms = po.MaterialSet([eos.Tillotson(name, eos.TILLOTSON[name]).as_material()])
        rho, u, reg = g[f"{name}_rho"], g[f"{name}_u"], g[f"{name}_region"]
        P = np.array([ms.eval(0, r, v)[0] for r, v in zip(rho, u)])
        want = tillotson_expected(g, name)
        pure = reg != TIL_BLEND
        rel = np.abs(P - want) / np.abs(want)
        assert np.max(rel[pure]) < 1e-14, (name, float(np.max(rel[pure])))
        scale = np.maximum(np.abs(g[f"{name}_P_co"]), np.abs(g[f"{name}_P_ex"]))
        assert np.max((np.abs(P - want) / scale)[~pure]) < 1e-13, name
