"""Seeded initial conditions for giant-impact runs.

The reference builds its bodies on a cubic lattice clipped to the layer radii
and thins the lattice to the requested particle count with a random removal
list (GI.h:35-445, create_removal_list GI.h:10-24), but seeds nothing and
places the impactor head-on (GI.h:597-600).  This generator keeps the
lattice-and-thin construction, draws every random choice from a
``numpy.random.Generator`` seeded by the caller, jitters the lattice, and
places the impactor on the two-body Kepler orbit that reaches contact with
the requested angle and speed.

Units are SI.  Particle masses are equal within a run (GI.h:325,386 give all
particles the same mass); ``h`` follows RealPtcl::initialize (class.h:196-199).
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

G = 6.67e-11
M_EARTH = 5.972e24

NFIELD = 34
FIELDS = [
    "x", "y", "z", "vx", "vy", "vz", "mass", "smth", "dens", "eng",
    "pres", "snds", "div_v", "rot_x", "rot_y", "rot_z", "bal", "ava", "grad_smth",
    "ax", "ay", "az", "eng_dot", "vhx", "vhy", "vhz", "eng_half", "dt",
    "gx", "gy", "gz", "pot", "ent", "temp",
]
FIELD = {n: i for i, n in enumerate(FIELDS)}


@dataclass
class Layer:
    material: int      # material index into the run's EoS list
    mass_frac: float   # fraction of the body's mass
    density: float     # uniform initial density [kg/m^3]


@dataclass
class Body:
    n: int
    mass: float
    layers: list       # innermost first


def _layer_radii(body: Body):
    radii = []
    vol = 0.0
    for L in body.layers:
        vol += body.mass * L.mass_frac / L.density
        radii.append((3.0 * vol / (4.0 * math.pi)) ** (1.0 / 3.0))
    return radii


def make_body(body: Body, rng: np.random.Generator, u0: float = 1.0e6):
    """Returns a field-major block [NFIELD, n] plus material ids for one body
    centred on the origin at rest."""
    radii = _layer_radii(body)
    m = body.mass / body.n
    counts = [int(round(body.n * L.mass_frac)) for L in body.layers]
    counts[-1] = body.n - sum(counts[:-1])
    pos_all, mat_all, dens_all = [], [], []
    r_in = 0.0
    for L, R, cnt in zip(body.layers, radii, counts):
        if cnt <= 0:
            r_in = R
            continue
        dx = (m / L.density) ** (1.0 / 3.0)
        # start slightly denser than the target spacing so the shell holds at least cnt points
        scale = 1.0
        while True:
            d = dx * 0.985 * scale
            k = int(math.ceil(R / d)) + 1
            ax = (np.arange(-k, k + 1) + 0.5 * (rng.random() - 0.5)) * d
            X, Y, Z = np.meshgrid(ax, ax, ax, indexing="ij")
            P = np.stack([X.ravel(), Y.ravel(), Z.ravel()], axis=1)
            P += (rng.random(P.shape) - 0.5) * (0.2 * d)          # lattice jitter, +-10% of the spacing
            r = np.sqrt((P * P).sum(axis=1))
            sel = P[(r < R) & (r >= r_in)]
            if len(sel) >= cnt:
                break
            scale *= 0.98
        keep = rng.choice(len(sel), size=cnt, replace=False)     # seeded removal list (GI.h:10-24)
        keep.sort()
        pos_all.append(sel[keep])
        mat_all.append(np.full(cnt, L.material, dtype=np.int32))
        dens_all.append(np.full(cnt, L.density))
        r_in = R
    pos = np.concatenate(pos_all)
    mats = np.concatenate(mat_all)
    dens = np.concatenate(dens_all)
    n = len(pos)
    F = np.zeros((NFIELD, n))
    F[FIELD["x"]], F[FIELD["y"]], F[FIELD["z"]] = pos.T
    F[FIELD["mass"]] = m
    F[FIELD["dens"]] = dens
    F[FIELD["eng"]] = u0
    F[FIELD["smth"]] = 1.2 * (m / dens) ** (1.0 / 3.0)   # class.h:196-199
    F[FIELD["grad_smth"]] = 1.0
    F[FIELD["bal"]] = 1.0                                 # RealPtcl() constructor, class.h:120-124
    F[FIELD["ava"]] = 1.0
    return F, mats, radii[-1]


def impact_geometry(Mt, Rt, Mi, Ri, angle_deg, v_over_vesc, sep_over_rt=4.0):
    """Relative position and velocity of the impactor with respect to the
    target so that the two-body orbit reaches contact (distance Rt + Ri) with
    speed v_over_vesc * v_esc and angle ``angle_deg`` from head-on."""
    mu = G * (Mt + Mi)
    rc = Rt + Ri
    vesc = math.sqrt(2.0 * mu / rc)
    vc = v_over_vesc * vesc
    th = math.radians(angle_deg)
    E = 0.5 * vc * vc - mu / rc
    Lz = rc * vc * math.sin(th)
    d = sep_over_rt * Rt
    vd = math.sqrt(max(2.0 * (E + mu / d), 0.0))
    vt = Lz / d
    vr = -math.sqrt(max(vd * vd - vt * vt, 0.0))
    return np.array([d, 0.0, 0.0]), np.array([vr, vt, 0.0]), vesc


def make_impact(n_target, n_impactor, m_target, m_impactor, layers_t, layers_i, angle_deg, v_over_vesc,
                seed, u0=1.0e6, sep_over_rt=4.0):
    """Two-body impact in the centre-of-mass frame.  Returns (F, ids, mats, info)."""
    rng = np.random.default_rng(seed)
    Ft, mt, Rt = make_body(Body(n_target, m_target, layers_t), rng, u0)
    Fi, mi, Ri = make_body(Body(n_impactor, m_impactor, layers_i), rng, u0)
    rel_p, rel_v, vesc = impact_geometry(m_target, Rt, m_impactor, Ri, angle_deg, v_over_vesc, sep_over_rt)
    Mtot = m_target + m_impactor
    # centre-of-mass frame
    pt = -rel_p * m_impactor / Mtot
    vt = -rel_v * m_impactor / Mtot
    pi_ = rel_p * m_target / Mtot
    vi = rel_v * m_target / Mtot
    for k, c in enumerate("xyz"):
        Ft[FIELD[c]] += pt[k]
        Fi[FIELD[c]] += pi_[k]
        Ft[FIELD["v" + c]] += vt[k]
        Fi[FIELD["v" + c]] += vi[k]
    F = np.concatenate([Ft, Fi], axis=1)
    mats = np.concatenate([mt, mi])
    ids = np.arange(F.shape[1], dtype=np.int64)
    info = {"R_target": Rt, "R_impactor": Ri, "v_esc": vesc, "separation": float(np.linalg.norm(rel_p)),
            "n_target": Ft.shape[1], "n_impactor": Fi.shape[1]}
    return F, ids, mats, info


# ---------------------------------------------------------------------------
# The workloads named by the benchmark configurations.

def config_small_impact(seed=1234, n_target=9000, n_impactor=1000):
    """10k-particle two-layer impact: iron core (30% of mass, 7800 kg/m^3) and
    granite mantle (2700 kg/m^3); 0.89 / 0.11 Earth masses; 45 degrees at
    1.0 v_esc from 4 target radii; analytic Tillotson iron (material 0) and
    granite (material 1)."""
    layers = [Layer(0, 0.3, 7800.0), Layer(1, 0.7, 2700.0)]
    return make_impact(n_target, n_impactor, 0.89 * M_EARTH, 0.11 * M_EARTH, layers, layers, 45.0, 1.0, seed)


def contact_separation(m_target, m_impactor, layers, overlap=0.0):
    """sep_over_rt that starts the impactor at contact: centre distance (1 - overlap) (R_t + R_i)
    in units of R_t (the layer radii of make_body's uniform-density shells)."""
    Rt = _layer_radii(Body(1, m_target, layers))[-1]
    Ri = _layer_radii(Body(1, m_impactor, layers))[-1]
    return (1.0 - overlap) * (Rt + Ri) / Rt


def config_1m_impact(seed=2024, n_target=900_000, n_impactor=100_000, angle=30.0, v=1.2, sep_over_rt=4.0):
    """1M-particle iron core / dunite mantle impact, 30 degrees at 1.2 v_esc from 4 target radii
    (``sep_over_rt``; contact_separation gives the bodies in contact); materials 0 = iron table,
    1 = dunite table (synthetic 200 x 200)."""
    layers = [Layer(0, 0.3, 7800.0), Layer(1, 0.7, 3320.0)]
    return make_impact(n_target, n_impactor, 0.89 * M_EARTH, 0.11 * M_EARTH, layers, layers, angle, v, seed,
                       sep_over_rt=sep_over_rt)


def config_1m_contact(seed=2024, n_target=900_000, n_impactor=100_000, overlap=0.02):
    """The 1M workload's bodies placed in contact (centres (1 - overlap) (R_t + R_i) apart) with the
    contact velocity of the 30 degree, 1.2 v_esc orbit: a state whose first steps shock the
    contact region (artificial viscosity and du/dt active)."""
    layers = [Layer(0, 0.3, 7800.0), Layer(1, 0.7, 3320.0)]
    sep = contact_separation(0.89 * M_EARTH, 0.11 * M_EARTH, layers, overlap)
    return config_1m_impact(seed, n_target, n_impactor, sep_over_rt=sep)


def config_4m_impact(seed=4096, n_target=3_600_000, n_impactor=400_000):
    """4M-particle three-layer impact: iron core, dunite mantle, granite crust
    (5% of mass); materials 0 iron, 1 dunite, 2 granite (synthetic tables)."""
    layers = [Layer(0, 0.3, 7800.0), Layer(1, 0.65, 3320.0), Layer(2, 0.05, 2700.0)]
    return make_impact(n_target, n_impactor, 0.89 * M_EARTH, 0.11 * M_EARTH, layers, layers, 45.0, 1.0, seed)


def sweep_draw(rng: np.random.Generator, n_lo: float, n_hi: float):
    """The random parameters of one sweep / serving impact, in draw order: (n_target, n_impactor,
    mass ratio, angle in degrees, speed in v_esc)."""
    n = int(round(np.exp(rng.uniform(np.log(n_lo), np.log(n_hi)))))
    q = float(rng.uniform(0.05, 0.5))
    angle = float(rng.uniform(0.0, 75.0))
    v = float(rng.uniform(1.0, 2.0))
    n_i = max(64, int(round(n * q / (1.0 + q))))
    n_t = max(64, n - n_i)
    return n_t, n_i, q, angle, v


def sweep_impact(rng: np.random.Generator, n_lo: float, n_hi: float, seed: int):
    """One impact of the batched sweep and of the serving stream: total particles
    log-uniform in [n_lo, n_hi], impactor / target mass ratio U[0.05, 0.5], impact
    angle U[0, 75] degrees, speed U[1, 2] v_esc; iron core (30%) / dunite mantle
    bodies of one Earth mass in total, equal-mass particles; materials 0 iron,
    1 dunite (the 1M workload's synthetic tables).  Returns (F, ids, mats, params)."""
    n_t, n_i, q, angle, v = sweep_draw(rng, n_lo, n_hi)
    layers = [Layer(0, 0.3, 7800.0), Layer(1, 0.7, 3320.0)]
    F, ids, mats, info = make_impact(n_t, n_i, M_EARTH / (1.0 + q), q * M_EARTH / (1.0 + q), layers, layers, angle, v,
                                     seed)
    return F, ids, mats, dict(n=int(F.shape[1]), mass_ratio=q, angle=angle, v_over_vesc=v, seed=seed)


def config_sweep(seed=3, n_runs=256, n_lo=5_000, n_hi=200_000):
    """The batched sweep: n_runs impacts drawn by sweep_impact from one seed."""
    rng = np.random.default_rng(seed)
    return [sweep_impact(rng, n_lo, n_hi, seed * 100_003 + k) for k in range(n_runs)]
