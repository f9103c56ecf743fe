"""The seeded initial-condition generator produces the bodies and orbits the workloads name.

The reference builds its bodies from a lattice thinned to the particle count (GI.h:35-445) with
unseeded randomness and a head-on approach (GI.h:597-600); the generator keeps the construction,
seeds it and places the impactor on the two-body orbit that reaches contact at the requested
angle and speed.  Checked here on the host: particle counts and masses, layer mass fractions and
densities, the centre-of-mass frame, the 4 R_t separation, and, from the two-body invariants of
the initial relative state, the speed (in units of v_esc) and the angle from head-on at contact."""
import math

import numpy as np
import pytest

from fdps_sph_gb300 import ic

F_ = ic.FIELD


def _bodies(F, info):
    nt = info["n_target"]
    return F[:, :nt], F[:, nt:]


def _com(B):
    m = B[F_["mass"]]
    return np.array([np.sum(m * B[F_[c]]) / np.sum(m) for c in "xyz"]), \
        np.array([np.sum(m * B[F_["v" + c]]) / np.sum(m) for c in "xyz"])


def _contact(F, info):
    """speed / v_esc and angle from head-on (degrees) when the two-body orbit of the bodies'
    centres of mass reaches contact (distance R_t + R_i)"""
    T, I = _bodies(F, info)
    Mt, Mi = T[F_["mass"]].sum(), I[F_["mass"]].sum()
    (xt, vt), (xi, vi) = _com(T), _com(I)
    r, v = xi - xt, vi - vt
    mu = ic.G * (Mt + Mi)
    E = 0.5 * v @ v - mu / np.linalg.norm(r)
    Lz = np.linalg.norm(np.cross(r, v))
    rc = info["R_target"] + info["R_impactor"]
    vc = math.sqrt(2.0 * (E + mu / rc))
    vesc = math.sqrt(2.0 * mu / rc)
    return vc / vesc, math.degrees(math.asin(min(1.0, Lz / (rc * vc)))), r, v


@pytest.mark.parametrize("which,n_t,n_i,m_t,m_i,angle,speed,layers", [
    ("small", 9000, 1000, 0.89, 0.11, 45.0, 1.0, [(0, 0.3, 7800.0), (1, 0.7, 2700.0)]),
    ("1m", 9000, 1000, 0.89, 0.11, 30.0, 1.2, [(0, 0.3, 7800.0), (1, 0.7, 3320.0)]),
    ("4m", 9000, 1000, 0.89, 0.11, 45.0, 1.0, [(0, 0.3, 7800.0), (1, 0.65, 3320.0), (2, 0.05, 2700.0)]),
])
def test_impact_configurations(which, n_t, n_i, m_t, m_i, angle, speed, layers):
    make = {"small": ic.config_small_impact, "1m": ic.config_1m_impact, "4m": ic.config_4m_impact}[which]
    F, ids, mats, info = make(n_target=n_t, n_impactor=n_i)
    assert F.shape == (ic.NFIELD, n_t + n_i) and info["n_target"] == n_t and info["n_impactor"] == n_i
    assert np.array_equal(ids, np.arange(n_t + n_i))
    T, I = _bodies(F, info)
    for B, M, nb in ((T, m_t, n_t), (I, m_i, n_i)):
        m = B[F_["mass"]]
        assert np.allclose(m, m[0]) and math.isclose(m.sum(), M * ic.M_EARTH, rel_tol=1e-12)
    mt = mats[:n_t]
    for mat, frac, dens in layers:   # layer mass fractions (equal-mass particles: count fractions)
        sel = mt == mat
        assert abs(np.mean(sel) - frac) <= 1.0 / n_t, (mat, np.mean(sel))
        assert np.all(T[F_["dens"]][sel] == dens)
    assert np.all(F[F_["eng"]] == 1.0e6)
    # h from RealPtcl::initialize (class.h:196-199)
    assert np.allclose(F[F_["smth"]], 1.2 * (F[F_["mass"]] / F[F_["dens"]]) ** (1.0 / 3.0), rtol=1e-14)
    # centre-of-mass frame (the bodies are placed by their lattice centres, which sit within a
    # fraction of a particle spacing of their centres of mass)
    m = F[F_["mass"]]
    for c in "xyz":
        assert abs(np.sum(m * F[F_[c]])) / m.sum() < 2e-3 * info["R_target"]
        assert abs(np.sum(m * F[F_["v" + c]])) / m.sum() < 1e-9 * info["v_esc"]
    # bodies inside their radii, separated by 4 target radii
    xt, _ = _com(T)
    xi, _ = _com(I)
    assert math.isclose(np.linalg.norm(xi - xt), 4.0 * info["R_target"], rel_tol=2e-3)
    rt = np.linalg.norm(np.stack([T[F_[c]] for c in "xyz"], 1) - xt, axis=1)
    assert rt.max() <= info["R_target"] * 1.003   # radius about the centre of mass (see above)
    # the orbit reaches contact at the requested speed and angle, approaching
    s, a, r, v = _contact(F, info)
    assert math.isclose(s, speed, rel_tol=2e-3), s
    assert abs(a - angle) < 0.3, a
    assert r @ v < 0.0


def test_contact_state_starts_at_contact():
    F, ids, mats, info = ic.config_1m_contact(n_target=9000, n_impactor=1000)
    T, I = _bodies(F, info)
    (xt, _), (xi, _) = _com(T), _com(I)
    assert math.isclose(np.linalg.norm(xi - xt), 0.98 * (info["R_target"] + info["R_impactor"]), rel_tol=2e-3)
    s, a, r, v = _contact(F, info)
    assert math.isclose(s, 1.2, rel_tol=2e-3) and abs(a - 30.0) < 0.3 and r @ v < 0.0


def test_generator_is_seeded():
    A = ic.config_small_impact(seed=5, n_target=900, n_impactor=100)[0]
    B = ic.config_small_impact(seed=5, n_target=900, n_impactor=100)[0]
    C = ic.config_small_impact(seed=6, n_target=900, n_impactor=100)[0]
    assert np.array_equal(A, B) and not np.array_equal(A, C)


def test_sweep_draws_stay_in_their_ranges():
    rng = np.random.default_rng(3)
    draws = [ic.sweep_draw(rng, 5_000, 200_000) for _ in range(2000)]
    n = np.array([d[0] + d[1] for d in draws])
    q = np.array([d[2] for d in draws])
    ang = np.array([d[3] for d in draws])
    v = np.array([d[4] for d in draws])
    assert n.min() >= 5_000 and n.max() <= 200_000
    # log-uniform: the median sits near the geometric mean of the range
    assert abs(np.log(np.median(n)) - 0.5 * (np.log(5e3) + np.log(2e5))) < 0.15
    assert q.min() >= 0.05 and q.max() <= 0.5 and ang.min() >= 0.0 and ang.max() <= 75.0
    assert v.min() >= 1.0 and v.max() <= 2.0
