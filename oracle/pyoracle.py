"""ctypes binding of the CPU oracle (test infrastructure only).

Only tests/, __graft_entry__.smoke() and bench.py's CPU-baseline leg import
this module.  It exposes the C restatement in oracle/sph_oracle.c over numpy
arrays in the same field-major particle layout the product library uses.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import build_oracle

NFIELD = 34
FIELDS = [
    "x", "y", "z", "vx", "vy", "vz", "mass", "smth", "dens", "eng",
    "pres", "snds", "div_v", "rot_x", "rot_y", "rot_z", "bal", "ava", "grad_smth",
    "ax", "ay", "az", "eng_dot", "vhx", "vhy", "vhz", "eng_half", "dt",
    "gx", "gy", "gz", "pot", "ent", "temp",
]
FIELD = {n: i for i, n in enumerate(FIELDS)}


class Material(C.Structure):
    _fields_ = [
        ("kind", C.c_int32), ("n_rho", C.c_int32), ("n_u", C.c_int32),
        ("rho", C.POINTER(C.c_double)), ("u", C.POINTER(C.c_double)),
        ("pres", C.POINTER(C.c_double)), ("snds", C.POINTER(C.c_double)),
        ("par", C.c_double * 10),
        ("temp", C.POINTER(C.c_double)), ("ent", C.POINTER(C.c_double)),
        ("line_rho", C.POINTER(C.c_double)), ("line_u", C.POINTER(C.c_double)),
    ]


class Config(C.Structure):
    _fields_ = [
        ("theta", C.c_double), ("n_leaf", C.c_int32), ("n_group", C.c_int32),
        ("n_dens_iter", C.c_int32), ("self_gravity", C.c_int32), ("ext_damp", C.c_int32),
        ("ext_damp_tend", C.c_double), ("damping", C.c_double), ("G", C.c_double),
        ("n_mat", C.c_int32), ("mat", C.POINTER(Material)),
        ("mode", C.c_int32), ("entropy_grid", C.c_int32), ("entropy_abs", C.c_int32),
        ("mantle_entropy", C.c_double), ("core_entropy", C.c_double),
    ]


class System(C.Structure):
    _fields_ = [
        ("n", C.c_int64), ("F", C.POINTER(C.c_double)), ("id", C.POINTER(C.c_int64)),
        ("mat", C.POINTER(C.c_int32)), ("time", C.c_double), ("dt", C.c_double), ("step", C.c_int64),
    ]


class RootBox(C.Structure):
    _fields_ = [("root_lo", C.c_double * 3), ("root_len", C.c_double), ("scale", C.c_double)]


class Cell(C.Structure):
    _fields_ = [
        ("start", C.c_int32), ("count", C.c_int32), ("level", C.c_int32), ("first_child", C.c_int32),
        ("n_child", C.c_int32), ("parent", C.c_int32),
        ("mass", C.c_double), ("mx", C.c_double), ("my", C.c_double), ("mz", C.c_double),
        ("com", C.c_double * 3), ("lo", C.c_double * 3), ("hi", C.c_double * 3), ("hmax", C.c_double),
    ]


class Tree(C.Structure):
    _fields_ = [
        ("n_cell", C.c_int64), ("cap", C.c_int64), ("c", C.POINTER(Cell)), ("rb", RootBox),
        ("keys", C.POINTER(C.c_uint64)),
    ]


_LIBS: dict[str, C.CDLL] = {}


def _p(a, t=C.c_double):
    return a.ctypes.data_as(C.POINTER(t))


def lib(fast: bool = False) -> C.CDLL:
    name = "liboracle_fast.so" if fast else "liboracle.so"
    if name not in _LIBS:
        build_oracle.build()
        L = C.CDLL(os.path.join(build_oracle.BUILD, name))
        L.or_kernel_W.restype = C.c_double
        L.or_kernel_W.argtypes = [C.c_double] * 4
        L.or_kernel_gradW.argtypes = [C.c_double] * 4 + [C.POINTER(C.c_double)]
        L.or_table_lookup.restype = C.c_double
        L.or_table_lookup.argtypes = [C.POINTER(C.c_double), C.c_int, C.POINTER(C.c_double), C.c_int,
                                      C.POINTER(C.c_double), C.c_double, C.c_double]
        L.or_eos_eval.argtypes = [C.POINTER(Material), C.c_double, C.c_double, C.POINTER(C.c_double),
                                  C.POINTER(C.c_double)]
        for f in ("or_eos_temperature", "or_eos_entropy"):
            getattr(L, f).restype = C.c_double
            getattr(L, f).argtypes = [C.POINTER(Material), C.c_double, C.c_double]
        L.or_eos_internal_energy.restype = C.c_double
        L.or_eos_internal_energy.argtypes = [C.POINTER(Material), C.c_double, C.c_double, C.c_int, C.c_int,
                                             C.POINTER(C.c_int)]
        L.or_entropy_step.restype = C.c_int64
        L.or_entropy_step.argtypes = [C.POINTER(System), C.POINTER(Config)]
        L.or_root_box.argtypes = [C.POINTER(C.c_double)] * 3 + [C.c_int64, C.POINTER(RootBox)]
        L.or_morton_keys.argtypes = [C.POINTER(C.c_double)] * 3 + [C.c_int64, C.POINTER(RootBox),
                                                                   C.POINTER(C.c_uint64)]
        L.or_sort_perm.argtypes = [C.POINTER(C.c_uint64), C.c_int64, C.POINTER(C.c_int64)]
        L.or_sort_system.argtypes = [C.POINTER(System), C.POINTER(Tree), C.c_int]
        L.or_tree_free.argtypes = [C.POINTER(Tree)]
        L.or_tree_groups.restype = C.c_int64
        L.or_tree_groups.argtypes = [C.POINTER(Tree), C.c_int, C.POINTER(C.c_int32)]
        L.or_sph_list.restype = C.c_int64
        L.or_sph_list.argtypes = [C.POINTER(Tree)] + [C.POINTER(C.c_double)] * 4 + [
            C.c_int64, C.c_int, C.POINTER(C.c_int32), C.c_int64]
        L.or_grav_list.argtypes = [C.POINTER(Tree)] + [C.POINTER(C.c_double)] * 3 + [
            C.c_int32, C.c_double, C.POINTER(C.c_int32), C.c_int64, C.POINTER(C.c_int64),
            C.POINTER(C.c_int32), C.c_int64, C.POINTER(C.c_int64)]
        for f in ("or_pass_density", "or_pass_gravity"):
            getattr(L, f).argtypes = [C.POINTER(System), C.POINTER(Tree), C.POINTER(Config)]
        for f in ("or_pass_derivative", "or_pass_hydro"):
            getattr(L, f).argtypes = [C.POINTER(System), C.POINTER(Tree)]
        L.or_pass_pressure.argtypes = [C.POINTER(System), C.POINTER(Config)]
        L.or_dt_global.restype = C.c_double
        L.or_dt_global.argtypes = [C.POINTER(System)]
        for f in ("or_compute_forces", "or_prologue"):
            getattr(L, f).argtypes = [C.POINTER(System), C.POINTER(Config)]
        L.or_step.argtypes = [C.POINTER(System), C.POINTER(Config), C.c_int]
        L.or_initialize_smth.argtypes = [C.POINTER(System)]
        L.or_num_threads.restype = C.c_int
        _LIBS[name] = L
    return _LIBS[name]


# --------------------------------------------------------------------------
# scalar helpers

def kernel_W(dx, dy, dz, h):
    return lib().or_kernel_W(dx, dy, dz, h)


def kernel_gradW(dx, dy, dz, h):
    g = (C.c_double * 3)()
    lib().or_kernel_gradW(dx, dy, dz, h, g)
    return np.array(g[:])


class MaterialSet:
    """Holds numpy buffers alive for a list of EoS materials."""

    def __init__(self, materials):
        self._keep = []
        arr = (Material * max(1, len(materials)))()
        for k, m in enumerate(materials):
            mm = arr[k]
            if m["kind"] == "table":
                rho = np.ascontiguousarray(m["rho"], dtype=np.float64)
                u = np.ascontiguousarray(m["u"], dtype=np.float64)
                P = np.ascontiguousarray(m["pres"], dtype=np.float64).reshape(-1)
                cs = np.ascontiguousarray(m["snds"], dtype=np.float64).reshape(-1)
                self._keep += [rho, u, P, cs]
                mm.kind = 0
                mm.n_rho, mm.n_u = len(rho), len(u)
                mm.rho, mm.u, mm.pres, mm.snds = _p(rho), _p(u), _p(P), _p(cs)
                if m.get("temp") is not None and m.get("ent") is not None:
                    T = np.ascontiguousarray(m["temp"], dtype=np.float64).reshape(-1)
                    S = np.ascontiguousarray(m["ent"], dtype=np.float64).reshape(-1)
                    lr = m.get("line_rho")
                    lu = m.get("line_u")
                    lr = np.repeat(rho, len(u)) if lr is None else np.ascontiguousarray(lr, np.float64).reshape(-1)
                    lu = np.tile(u, len(rho)) if lu is None else np.ascontiguousarray(lu, np.float64).reshape(-1)
                    self._keep += [T, S, lr, lu]
                    mm.temp, mm.ent, mm.line_rho, mm.line_u = _p(T), _p(S), _p(lr), _p(lu)
            elif m["kind"] == "tillotson":
                mm.kind = 1
                for q, v in enumerate(m["par"]):
                    mm.par[q] = float(v)
            elif m["kind"] == "ideal":
                mm.kind = 2
                mm.par[0] = float(m["gamma"])
            else:
                raise ValueError(m["kind"])
        self.arr = arr
        self.n = len(materials)

    def eval(self, k, rho, u):
        P = C.c_double()
        cs = C.c_double()
        lib().or_eos_eval(C.byref(self.arr[k]), float(rho), float(u), C.byref(P), C.byref(cs))
        return P.value, cs.value

    def temperature(self, k, rho, u):
        return lib().or_eos_temperature(C.byref(self.arr[k]), float(rho), float(u))

    def entropy(self, k, rho, u):
        return lib().or_eos_entropy(C.byref(self.arr[k]), float(rho), float(u))

    def internal_energy(self, k, rho, s, grid=120, abs_mode=0):
        """(u, undefined) of RestrictedBilinearInterpolation (literal O(lines) scans)"""
        undef = C.c_int()
        u = lib().or_eos_internal_energy(C.byref(self.arr[k]), float(rho), float(s), int(grid), int(abs_mode),
                                         C.byref(undef))
        return u, bool(undef.value)


def make_config(materials: MaterialSet, theta=0.5, n_leaf=8, n_group=256, n_dens_iter=4, self_gravity=True,
                ext_damp=False, ext_damp_tend=5000.0, damping=1.0, G=6.67e-11, mode=1,
                mantle_entropy=3.12432609e3, core_entropy=3.12432609e3, entropy_grid=120,
                entropy_abs=0) -> Config:
    cfg = Config()
    cfg.theta = theta
    cfg.n_leaf = n_leaf
    cfg.n_group = n_group
    cfg.n_dens_iter = n_dens_iter
    cfg.self_gravity = int(bool(self_gravity))
    cfg.ext_damp = int(bool(ext_damp))
    cfg.ext_damp_tend = ext_damp_tend
    cfg.damping = damping
    cfg.G = G
    cfg.n_mat = materials.n
    cfg.mat = C.cast(materials.arr, C.POINTER(Material))
    cfg.mode = mode
    cfg.mantle_entropy = mantle_entropy
    cfg.core_entropy = core_entropy
    cfg.entropy_grid = entropy_grid
    cfg.entropy_abs = entropy_abs
    cfg._materials = materials  # keep alive
    return cfg


class OracleSystem:
    """Field-major particle block owned by numpy, viewed by the C oracle."""

    def __init__(self, fields: np.ndarray, ids: np.ndarray, mats: np.ndarray, time=0.0, dt=0.0, step=0,
                 fast=False):
        n = fields.shape[1]
        assert fields.shape == (NFIELD, n)
        self.F = np.ascontiguousarray(fields, dtype=np.float64).copy()
        self.id = np.ascontiguousarray(ids, dtype=np.int64).copy()
        self.mat = np.ascontiguousarray(mats, dtype=np.int32).copy()
        self.sys = System(n, _p(self.F), _p(self.id, C.c_int64), _p(self.mat, C.c_int32), time, dt, step)
        self.lib = lib(fast)

    @property
    def n(self):
        return self.F.shape[1]

    def field(self, name):
        return self.F[FIELD[name]]

    def prologue(self, cfg):
        rc = self.lib.or_prologue(C.byref(self.sys), C.byref(cfg))
        if rc != 0:
            raise RuntimeError("oracle prologue failed")

    def step(self, cfg, n_steps=1):
        rc = self.lib.or_step(C.byref(self.sys), C.byref(cfg), int(n_steps))
        if rc == -2:
            raise RuntimeError("oracle step: a mode-2 energy lookup is undefined or non-finite")
        if rc != 0:
            raise RuntimeError("oracle step failed")

    def entropy_step(self, cfg):
        """SetConstantEntropy + CalcAll on the current state; returns the undefined / non-finite count"""
        return int(self.lib.or_entropy_step(C.byref(self.sys), C.byref(cfg)))

    def compute_forces(self, cfg):
        if self.lib.or_compute_forces(C.byref(self.sys), C.byref(cfg)) != 0:
            raise RuntimeError("oracle compute_forces failed")

    def initialize_smth(self):
        self.lib.or_initialize_smth(C.byref(self.sys))

    def by_id(self):
        """Fields reordered by particle id (ascending)."""
        o = np.argsort(self.id, kind="stable")
        return self.F[:, o], self.id[o], self.mat[o]


class OracleTree:
    """Sorts an OracleSystem by Morton key and builds the oracle octree."""

    def __init__(self, system: OracleSystem, n_leaf=8):
        self.system = system
        self.tree = Tree()
        self.lib = system.lib
        if self.lib.or_sort_system(C.byref(system.sys), C.byref(self.tree), n_leaf) != 0:
            raise RuntimeError("tree build failed")

    def __del__(self):
        try:
            self.lib.or_tree_free(C.byref(self.tree))
        except Exception:
            pass

    @property
    def n_cell(self):
        return self.tree.n_cell

    def cells(self):
        n = self.tree.n_cell
        out = np.ctypeslib.as_array(self.tree.c, shape=(n,))
        return out.copy()

    def keys(self):
        return np.ctypeslib.as_array(self.tree.keys, shape=(self.system.n,)).copy()

    def groups(self, n_group):
        buf = np.zeros(max(1, self.tree.n_cell), dtype=np.int32)
        k = self.lib.or_tree_groups(C.byref(self.tree), n_group, _p(buf, C.c_int32))
        return buf[:k].copy()

    def sph_list(self, i, mode):
        s = self.system
        cap = 4096
        out = np.zeros(cap, dtype=np.int32)
        k = self.lib.or_sph_list(C.byref(self.tree), _p(s.field("x")), _p(s.field("y")), _p(s.field("z")),
                                 _p(s.field("smth")), int(i), int(mode), _p(out, C.c_int32), cap)
        if k > cap:
            out = np.zeros(k, dtype=np.int32)
            self.lib.or_sph_list(C.byref(self.tree), _p(s.field("x")), _p(s.field("y")), _p(s.field("z")),
                                 _p(s.field("smth")), int(i), int(mode), _p(out, C.c_int32), k)
        return out[:k].copy()

    def grav_list(self, gcell, theta):
        s = self.system
        ne, ns = C.c_int64(), C.c_int64()
        cap = 1 << 16
        epj = np.zeros(cap, dtype=np.int32)
        spj = np.zeros(cap, dtype=np.int32)
        self.lib.or_grav_list(C.byref(self.tree), _p(s.field("x")), _p(s.field("y")), _p(s.field("z")),
                              int(gcell), float(theta), _p(epj, C.c_int32), cap, C.byref(ne),
                              _p(spj, C.c_int32), cap, C.byref(ns))
        if ne.value > cap or ns.value > cap:
            cap = max(ne.value, ns.value)
            epj = np.zeros(cap, dtype=np.int32)
            spj = np.zeros(cap, dtype=np.int32)
            self.lib.or_grav_list(C.byref(self.tree), _p(s.field("x")), _p(s.field("y")), _p(s.field("z")),
                                  int(gcell), float(theta), _p(epj, C.c_int32), cap, C.byref(ne),
                                  _p(spj, C.c_int32), cap, C.byref(ns))
        return epj[:ne.value].copy(), spj[:ns.value].copy()

    def pass_density(self, cfg):
        self.lib.or_pass_density(C.byref(self.system.sys), C.byref(self.tree), C.byref(cfg))

    def pass_pressure(self, cfg):
        self.lib.or_pass_pressure(C.byref(self.system.sys), C.byref(cfg))

    def pass_derivative(self):
        self.lib.or_pass_derivative(C.byref(self.system.sys), C.byref(self.tree))

    def pass_hydro(self):
        self.lib.or_pass_hydro(C.byref(self.system.sys), C.byref(self.tree))

    def pass_gravity(self, cfg):
        self.lib.or_pass_gravity(C.byref(self.system.sys), C.byref(self.tree), C.byref(cfg))


def _bind_integrator(L):
    L.or_kick_drift_predict.argtypes = [C.POINTER(System), C.c_double]
    L.or_final_kick.argtypes = [C.POINTER(System), C.c_double, C.c_double]


def kick_drift_predict(system: "OracleSystem", dt: float):
    _bind_integrator(system.lib)
    system.lib.or_kick_drift_predict(C.byref(system.sys), float(dt))


def final_kick(system: "OracleSystem", dt: float, damping: float):
    _bind_integrator(system.lib)
    system.lib.or_final_kick(C.byref(system.sys), float(dt), float(damping))


def dt_global(system: "OracleSystem") -> float:
    return system.lib.or_dt_global(C.byref(system.sys))
