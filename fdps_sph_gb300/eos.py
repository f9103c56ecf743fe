"""Equation-of-state data: the reference's ``rho_u`` table format and the
analytic Tillotson parameter sets.

Table format (reader: EoS.h:121-221 / 290-390; writer:
eos/ANEOS_conversion.py:157-164): a header line ``#  n_rho n_u ...``, a
column-name comment, then ``n_rho * n_u`` rows of six columns
``rho u T P c_s S`` with rho the outer (slow) index.  The density axis is
column 0 of the first row of each density block; the energy axis is column 1
of the first density block; pressure is column 3 and sound speed column 4
(EoS.h:218-221, 241-247, 394-400).
"""
from __future__ import annotations

import math
import os
from dataclasses import dataclass, field

import numpy as np

# Tillotson parameters (rho0 [kg/m^3], u0, uiv, ucv [J/kg], A, B [Pa], a, b, alpha, beta).
# Granite: EoS.h:446.  Iron: EoS.h:448 (commented out in the reference, used here for the
# analytic mode).  "dunite-like" is a synthetic parameter set chosen by this project for the
# synthetic tables (dunite reference density with basalt-type a, b, alpha, beta); it is not a
# published fit.
TILLOTSON = {
    "granite": (2680.0, 16.0e6, 3.5e6, 18.00e6, 18.0e9, 18.0e9, 0.5, 1.3, 5.0, 5.0),
    "iron": (7800.0, 9.5e6, 2.4e6, 8.67e6, 128.0e9, 105.0e9, 0.5, 1.5, 5.0, 5.0),
    "dunite": (3320.0, 487.0e6, 4.72e6, 18.2e6, 131.0e9, 49.0e9, 0.5, 1.5, 5.0, 5.0),
}


@dataclass
class Table:
    """A density x energy table: axes plus the pressure and sound-speed planes."""

    rho: np.ndarray
    u: np.ndarray
    pres: np.ndarray  # [n_rho, n_u]
    snds: np.ndarray  # [n_rho, n_u]
    temp: np.ndarray | None = None
    ent: np.ndarray | None = None
    name: str = ""
    line_rho: np.ndarray | None = None   # column 0 of every line, file order (None: the axis repeated)
    line_u: np.ndarray | None = None     # column 1 of every line

    def as_material(self) -> dict:
        return {"kind": "table", "rho": self.rho, "u": self.u, "pres": self.pres, "snds": self.snds,
                "temp": self.temp, "ent": self.ent, "line_rho": self.line_rho, "line_u": self.line_u}


@dataclass
class IdealGas:
    """EoS::IdealGas (EoS.h:37-66): P = (gamma - 1) rho u, c_s = sqrt(gamma (gamma - 1) u)."""
    gamma: float

    def as_material(self) -> dict:
        return {"kind": "ideal", "gamma": self.gamma}


@dataclass
class Tillotson:
    name: str
    par: tuple = field(default_factory=tuple)

    def as_material(self) -> dict:
        return {"kind": "tillotson", "par": self.par}


def read_rho_u(path: str) -> Table:
    """Read a ``rho_u`` table the way EoS.h:121-221 does (header line, comment
    lines skipped, ``n_u`` rows per density block)."""
    with open(path, "r") as fh:
        lines = fh.readlines()
    if not lines:
        raise ValueError(f"{path}: empty EoS table")
    head = lines[0].split()
    if len(head) < 3 or head[0] != "#":
        raise ValueError(f"{path}: first line must be '#  n_rho n_u'")
    n_rho, n_u = int(head[1]), int(head[2])
    rows = []
    for ln in lines[1:]:
        if ln.startswith("#"):
            continue
        parts = ln.split()
        if not parts:
            continue
        rows.append([float(v) for v in parts[:6]])
    data = np.array(rows, dtype=np.float64)
    if data.shape != (n_rho * n_u, 6):
        raise ValueError(f"{path}: expected {n_rho * n_u} rows of 6 columns, found {data.shape}")
    data = data.reshape(n_rho, n_u, 6)
    rho = data[:, 0, 0].copy()
    u = data[0, :, 1].copy()
    if np.any(np.diff(rho) <= 0) or np.any(np.diff(u) <= 0):
        raise ValueError(f"{path}: axes must be strictly ascending")
    return Table(rho=rho, u=u, temp=data[:, :, 2].copy(), pres=data[:, :, 3].copy(),
                 snds=data[:, :, 4].copy(), ent=data[:, :, 5].copy(), name=os.path.basename(path),
                 line_rho=data[:, :, 0].reshape(-1).copy(), line_u=data[:, :, 1].reshape(-1).copy())


def write_rho_u(path: str, t: Table) -> None:
    """Write a table in the format of eos/ANEOS_conversion.py:157-164."""
    n_rho, n_u = len(t.rho), len(t.u)
    temp = t.temp if t.temp is not None else np.zeros((n_rho, n_u))
    ent = t.ent if t.ent is not None else np.zeros((n_rho, n_u))
    with open(path, "w") as fh:
        fh.write("%s %i %i %s \n" % ("# ", n_rho, n_u, ":Grid numbers for density and internal energy"))
        fh.write("# Density (km/m3), Internal energy (kJ/kg), Temperature (K), Pressure (Pa), "
                 "Sound speed (m/s), Entropy (J/K/kg) \n")
        for m in range(n_rho):
            for k in range(n_u):
                fh.write("%15.8E %15.8E %15.8E  %15.8E %15.8E %15.8E \n" % (
                    t.rho[m], t.u[k], temp[m, k], t.pres[m, k], t.snds[m, k], ent[m, k]))


def tillotson_eval(par, rho, u):
    """Vectorised analytic Tillotson P and c_s: the generator of the synthetic tables.  The
    oracle's or_tillotson and the device EoS evaluate the same formulas in the reference's
    operation order (P_co / P_ex, EoS.h:91-103); this one keeps the order the committed
    synthetic-table fixtures were made with (the two agree to a few ulps)."""
    rho0, u0, uiv, ucv, A, B, a, b, alpha, beta = par
    rho = np.asarray(rho, dtype=np.float64)
    u = np.asarray(u, dtype=np.float64)
    eta = rho / rho0
    mu = eta - 1.0
    om = u / (u0 * eta * eta) + 1.0
    Pc = (a + b / om) * rho * u + A * mu + B * mu * mu
    dPc_r = (a + b / om) * u + 2.0 * b * u * (om - 1.0) / (om * om) + (A + 2.0 * B * mu) / rho0
    dPc_u = (a + b / om) * rho - rho * b * (om - 1.0) / (om * om)
    z = rho0 / rho - 1.0
    E1 = np.exp(-alpha * z)
    E2 = np.exp(-beta * z * z)
    Q = b * rho * u / om + A * mu * E1
    Pe = a * rho * u + Q * E2
    dQ = b * u / om + 2.0 * b * u * (om - 1.0) / (om * om) + A / rho0 * E1 + A * mu * alpha * E1 * (z + 1.0) / rho
    dPe_r = a * u + dQ * E2 + Q * 2.0 * beta * z * (z + 1.0) * E2 / rho
    dPe_u = a * rho + E2 * (b * rho / om - b * rho * (om - 1.0) / (om * om))
    w = ucv - uiv
    Pm = ((u - uiv) * Pe + (ucv - u) * Pc) / w
    dPm_r = ((u - uiv) * dPe_r + (ucv - u) * dPc_r) / w
    dPm_u = (Pe - Pc + (u - uiv) * dPe_u + (ucv - u) * dPc_u) / w
    comp = (rho >= rho0) | (u <= uiv)
    hot = (~comp) & (u >= ucv)
    P = np.where(comp, Pc, np.where(hot, Pe, Pm))
    dr = np.where(comp, dPc_r, np.where(hot, dPe_r, dPm_r))
    du = np.where(comp, dPc_u, np.where(hot, dPe_u, dPm_u))
    c2 = dr + P / (rho * rho) * du
    c2 = np.where(c2 > 1.0e-2 * A / rho0, c2, 1.0e-2 * A / rho0)
    return P, np.sqrt(c2)


def synthetic_table(material: str, n_rho: int = 200, n_u: int = 200, rho_range=(1.0e1, 3.0e4),
                    u_range=(1.0e3, 1.0e9)) -> Table:
    """Synthetic 'ANEOS-like' table: log-spaced density and energy axes, P and
    c_s from the analytic Tillotson parameters of ``material``.  Temperature
    is u / (1000 J/kg/K) and entropy 1000 ln(u / 1000) - 287 ln(rho / 1000)
    (rising with u at fixed rho); both are read only by mode 2.  Every column
    is rounded through the text format, so a written-then-read table is
    bit-identical."""
    par = TILLOTSON[material]
    rho = np.geomspace(rho_range[0], rho_range[1], n_rho)
    u = np.geomspace(u_range[0], u_range[1], n_u)
    # round the axes through the text format so a written-then-read table is bit-identical
    rho = np.array([float("%15.8E" % v) for v in rho])
    u = np.array([float("%15.8E" % v) for v in u])
    R, U = np.meshgrid(rho, u, indexing="ij")
    P, cs = tillotson_eval(par, R, U)
    P = np.vectorize(lambda v: float("%15.8E" % v))(P)
    cs = np.vectorize(lambda v: float("%15.8E" % v))(cs)
    temp = np.vectorize(lambda v: float("%15.8E" % v))(U / 1.0e3)
    ent = np.vectorize(lambda v: float("%15.8E" % v))(1.0e3 * np.log(U / 1.0e3) - 287.0 * np.log(R / 1.0e3))
    return Table(rho=rho, u=u, pres=P, snds=cs, temp=temp, ent=ent, name=f"synthetic-{material}")


def material_for(spec: str):
    """'tillotson:iron', 'table:/path/file.rho_u.txt', 'synthetic:dunite' -> material object."""
    kind, _, arg = spec.partition(":")
    if kind == "tillotson":
        return Tillotson(arg, TILLOTSON[arg])
    if kind == "table":
        return read_rho_u(arg)
    if kind == "synthetic":
        return synthetic_table(arg)
    raise ValueError(spec)


def _rel(a, b):
    return abs(a - b) / max(abs(b), 1e-300)


if __name__ == "__main__":  # quick self-check of the analytic branches
    for name, p in TILLOTSON.items():
        P, c = tillotson_eval(p, np.array([p[0] * 1.1, p[0] * 0.8, p[0] * 0.5]), np.array([1e6, 1e7, 1e8]))
        print(name, P, c)
    print(math.pi)
