"""ctypes binding of libsph_gb300.so (the C ABI declared in include/sph_gb300.h).

The product path: every call here goes to the CUDA library; there is no CPU
fallback.  If the library is missing or no GPU is present, calls raise.
"""
from __future__ import annotations

import ctypes as C
import os

import numpy as np

from . import layouts as T

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "libsph_gb300.so")

NFIELD = 34
FIELDS = [
    "x", "y", "z", "vx", "vy", "vz", "mass", "smth", "dens", "eng",
    "pres", "snds", "div_v", "rot_x", "rot_y", "rot_z", "bal", "ava", "grad_smth",
    "ax", "ay", "az", "eng_dot", "vhx", "vhy", "vhz", "eng_half", "dt",
    "gx", "gy", "gz", "pot", "ent", "temp",
]
FIELD = {n: i for i, n in enumerate(FIELDS)}

SPH_OK = 0
ERRORS = {-1: "SPH_ERR_ARG", -2: "SPH_ERR_CUDA", -3: "SPH_ERR_OOM", -4: "SPH_ERR_TABLE", -5: "SPH_ERR_NONFINITE",
          -6: "SPH_ERR_CAPACITY", -7: "SPH_ERR_STATE", -8: "SPH_ERR_TIMEOUT"}
SPH_ERR_ARG, SPH_ERR_STATE = -1, -7
PREC_FP64 = 0
PREC_MIXED = 1

EXPORTS = [
    "sph_dispatch_dens", "sph_retrieve_dens", "sph_dispatch_drvt", "sph_retrieve_drvt",
    "sph_dispatch_hydro", "sph_retrieve_hydro", "sph_dispatch_grav", "sph_retrieve_grav",
    "sph_batch_last_error", "sph_config_default", "sph_ctx_create", "sph_ctx_destroy", "sph_last_error",
    "sph_set_eos_table", "sph_load_eos_table_file", "sph_set_eos_tillotson", "sph_upload", "sph_download",
    "sph_prologue", "sph_step", "sph_get_time", "sph_diagnostics", "sph_run_pass", "sph_get_order",
    "sph_get_neighbors", "sph_get_tree", "sph_get_grav_list", "sph_get_timings", "sph_step_timed",
    "sph_get_counters", "sph_probe_peak", "sph_morton_order_noalloc",
    "sph_add_run", "sph_remove_run", "sph_list_runs", "sph_run_info", "sph_download_run", "sph_run_diagnostics",
    "sph_autotune", "sph_set_eos_ideal", "sph_set_eos_entropy", "sph_eos_eval", "sph_download_fields",
    "sph_step_download", "sph_read_eos_table_file", "sph_read_eos_table_error", "sph_get_grav_lists",
    "sph_batch_set_precision", "sph_batch_set_staging", "sph_dispatch_index_dens", "sph_dispatch_index_drvt",
    "sph_dispatch_index_hydro", "sph_dispatch_index_grav",
]
# fields a step reads or carries unchanged (SPH_STEP_INPUT_FIELDS): what SPH_UPLOAD_STEP_INPUTS copies
STEP_INPUT_FIELDS = ["x", "y", "z", "vx", "vy", "vz", "mass", "smth", "eng", "ava", "ax", "ay", "az", "eng_dot",
                     "gx", "gy", "gz", "ent", "temp"]
# fields a step writes (SPH_STEP_OUTPUT_FIELDS; mode 2 adds ent and temp)
STEP_OUTPUT_FIELDS = [f for f in FIELDS if f not in ("mass", "ava", "ent", "temp")]
EOS_QUANTITY = {"pressure": 0, "sound_speed": 1, "temperature": 2, "entropy": 3, "internal_energy": 4}
ENTROPY_ABS_INT = 0
ENTROPY_ABS_REAL = 1
NOALLOC_MAX_N = 131072
SEGMENTS = ["kdp", "tree", "dens_list", "dens", "eos", "drvt_list", "drvt", "hydro_list", "hydro", "grav_list",
            "grav", "final", "sort", "nbr_prep", "entropy"]


class SphError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"{ERRORS.get(code, code)}: {msg}")
        self.code = code


class Config(C.Structure):
    _fields_ = [
        ("theta", C.c_double), ("n_leaf", C.c_int32), ("n_group", C.c_int32), ("n_dens_iter", C.c_int32),
        ("self_gravity", C.c_int32), ("ext_damp", C.c_int32), ("precision", C.c_int32),
        ("ext_damp_tend", C.c_double), ("damping", C.c_double), ("G", C.c_double), ("device", C.c_int32),
        ("mode", C.c_int32), ("mantle_entropy", C.c_double), ("core_entropy", C.c_double),
        ("entropy_grid", C.c_int32), ("entropy_abs", C.c_int32),
    ]


_lib = None


def load() -> C.CDLL:
    """Loads the in-tree library (built by fdps_sph_gb300.build)."""
    global _lib
    if _lib is not None:
        return _lib
    if not os.path.exists(LIB_PATH):
        raise RuntimeError(f"{LIB_PATH} is missing: run fdps_sph_gb300.build.build() (nvcc, sm_103a)")
    L = C.CDLL(LIB_PATH)
    P = C.c_void_p
    i32p = C.POINTER(C.c_int)
    for k in ("dens", "drvt", "hydro"):
        getattr(L, f"sph_dispatch_{k}").argtypes = [C.c_int, C.c_int, P, i32p, P, i32p]
        getattr(L, f"sph_retrieve_{k}").argtypes = [C.c_int, C.c_int, i32p, P]
    L.sph_dispatch_grav.argtypes = [C.c_int, C.c_int, P, i32p, P, i32p, P, i32p]
    for k in ("dens", "drvt", "hydro"):
        getattr(L, f"sph_dispatch_index_{k}").argtypes = [C.c_int, C.c_int, P, i32p, P, i32p, P, C.c_int, C.c_int]
    L.sph_dispatch_index_grav.argtypes = [C.c_int, C.c_int, P, i32p, P, i32p, P, i32p, P, C.c_int, P, C.c_int,
                                          C.c_int]
    L.sph_retrieve_grav.argtypes = [C.c_int, C.c_int, i32p, P]
    L.sph_batch_last_error.restype = C.c_char_p
    L.sph_batch_set_precision.argtypes = [C.c_int]
    L.sph_batch_set_staging.argtypes = [C.c_int]
    L.sph_config_default.argtypes = [C.POINTER(Config)]
    L.sph_config_default.restype = None
    L.sph_ctx_create.argtypes = [C.POINTER(Config), C.POINTER(C.c_void_p)]
    L.sph_ctx_destroy.argtypes = [P]
    L.sph_last_error.argtypes = [P]
    L.sph_last_error.restype = C.c_char_p
    L.sph_set_eos_table.argtypes = [P, C.c_int, P, C.c_int, P, C.c_int, P, P]
    L.sph_load_eos_table_file.argtypes = [P, C.c_int, C.c_char_p]
    L.sph_read_eos_table_file.argtypes = [C.c_char_p, i32p, i32p, P, P, P, i32p]
    L.sph_read_eos_table_error.restype = C.c_char_p
    L.sph_set_eos_tillotson.argtypes = [P, C.c_int, P]
    L.sph_set_eos_ideal.argtypes = [P, C.c_int, C.c_double]
    L.sph_set_eos_entropy.argtypes = [P, C.c_int, P, P, P, P]
    L.sph_eos_eval.argtypes = [P, C.c_int, C.c_int, C.c_int64, P, P, P, C.POINTER(C.c_int64)]
    L.sph_upload.argtypes = [P, C.c_int64, P, C.c_int64, P, P, C.c_double, C.c_double, C.c_int]
    L.sph_step_timed.argtypes = [P, C.c_int, C.POINTER(C.c_double)]
    L.sph_get_counters.argtypes = [P, P]
    L.sph_probe_peak.argtypes = [C.c_int, C.c_int, C.POINTER(C.c_double)]
    L.sph_morton_order_noalloc.argtypes = [P, P, P, C.c_int64, P, P, P]
    L.sph_download.argtypes = [P, P, C.c_int64, P, P]
    L.sph_download_fields.argtypes = [P, P, C.c_int64, C.c_uint64, P, P]
    L.sph_step_download.argtypes = [P, P, C.c_int64, C.c_uint64]
    L.sph_prologue.argtypes = [P]
    L.sph_step.argtypes = [P, C.c_int]
    L.sph_get_time.argtypes = [P, C.POINTER(C.c_double), C.POINTER(C.c_double), C.POINTER(C.c_int64)]
    L.sph_diagnostics.argtypes = [P, P]
    L.sph_run_pass.argtypes = [P, C.c_int]
    L.sph_get_order.argtypes = [P, P, P]
    L.sph_get_neighbors.argtypes = [P, C.c_int, C.c_int64, P, C.c_int64, C.POINTER(C.c_int64)]
    L.sph_get_tree.argtypes = [P, C.POINTER(C.c_int64), P, P, P, P, P]
    L.sph_get_grav_list.argtypes = [P, C.c_int64, C.POINTER(C.c_int64), P, C.c_int64, C.POINTER(C.c_int64), P, P,
                                    C.c_int64, C.POINTER(C.c_int64), P, P]
    L.sph_get_timings.argtypes = [P, P, C.c_int, C.POINTER(C.c_int)]
    L.sph_add_run.argtypes = [P, C.c_int64, P, C.c_int64, P, P, C.c_double, C.c_double, C.c_int,
                              C.POINTER(C.c_int64)]
    L.sph_remove_run.argtypes = [P, C.c_int64]
    L.sph_list_runs.argtypes = [P, P, C.c_int, C.POINTER(C.c_int)]
    L.sph_run_info.argtypes = [P, C.c_int64, C.POINTER(C.c_int64), C.POINTER(C.c_double), C.POINTER(C.c_double),
                               C.POINTER(C.c_int64)]
    L.sph_download_run.argtypes = [P, C.c_int64, P, C.c_int64, P, P]
    L.sph_run_diagnostics.argtypes = [P, C.c_int64, P]
    L.sph_autotune.argtypes = [P, C.c_int, P]
    i64p = C.POINTER(C.c_int64)
    L.sph_get_grav_lists.argtypes = [P, i64p, i64p, i64p, P, P, P, P, P, P, P, P]
    _lib = L
    return L


def _ptr(a):
    return None if a is None else a.ctypes.data_as(C.c_void_p)


def read_table_file(path: str):
    """A rho-u table file read by the library's reader (sph_read_eos_table_file: host only, the
    reader sph_load_eos_table_file uses).  Returns (rho axis, u axis, columns [6, n_rho * n_u],
    number of columns in the file)."""
    L = load()
    nr, nu, nc = C.c_int(), C.c_int(), C.c_int()
    rc = L.sph_read_eos_table_file(path.encode(), C.byref(nr), C.byref(nu), None, None, None, C.byref(nc))
    if rc != SPH_OK:
        raise SphError(rc, L.sph_read_eos_table_error().decode())
    rho = np.empty(nr.value)
    u = np.empty(nu.value)
    cols = np.empty((6, nr.value * nu.value))
    rc = L.sph_read_eos_table_file(path.encode(), C.byref(nr), C.byref(nu), _ptr(rho), _ptr(u), _ptr(cols), None)
    if rc != SPH_OK:
        raise SphError(rc, L.sph_read_eos_table_error().decode())
    return rho, u, cols, nc.value


def default_config(**kw) -> Config:
    cfg = Config()
    load().sph_config_default(C.byref(cfg))
    for k, v in kw.items():
        if k == "precision" and isinstance(v, str):
            v = {"fp64": PREC_FP64, "mixed": PREC_MIXED}[v]
        setattr(cfg, k, v)
    return cfg


class Context:
    """A device-resident run: C ABI context owning the particle state in HBM."""

    def __init__(self, config: Config | None = None, **kw):
        self.L = load()
        cfg = config if config is not None else default_config(**kw)
        h = C.c_void_p()
        rc = self.L.sph_ctx_create(C.byref(cfg), C.byref(h))
        if rc != SPH_OK:
            raise SphError(rc, "sph_ctx_create failed (no CUDA device?)")
        self.h = h
        self.cfg = cfg
        self.n = 0

    def close(self):
        if getattr(self, "h", None):
            self.L.sph_ctx_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != SPH_OK:
            raise SphError(rc, self.L.sph_last_error(self.h).decode())

    # EoS ------------------------------------------------------------------
    def set_material(self, k: int, mat):
        d = mat.as_material() if hasattr(mat, "as_material") else mat
        if d["kind"] == "table":
            rho = np.ascontiguousarray(d["rho"], np.float64)
            u = np.ascontiguousarray(d["u"], np.float64)
            P = np.ascontiguousarray(d["pres"], np.float64)
            cs = np.ascontiguousarray(d["snds"], np.float64)
            self._check(self.L.sph_set_eos_table(self.h, k, _ptr(rho), len(rho), _ptr(u), len(u), _ptr(P), _ptr(cs)))
            if d.get("temp") is not None and d.get("ent") is not None:
                Tp = np.ascontiguousarray(d["temp"], np.float64)
                Sp = np.ascontiguousarray(d["ent"], np.float64)
                lr = d.get("line_rho")
                lu = d.get("line_u")
                lr = None if lr is None else np.ascontiguousarray(lr, np.float64)
                lu = None if lu is None else np.ascontiguousarray(lu, np.float64)
                self._check(self.L.sph_set_eos_entropy(self.h, k, _ptr(Tp), _ptr(Sp), _ptr(lr), _ptr(lu)))
        elif d["kind"] == "tillotson":
            par = np.ascontiguousarray(d["par"], np.float64)
            self._check(self.L.sph_set_eos_tillotson(self.h, k, _ptr(par)))
        elif d["kind"] == "ideal":
            self._check(self.L.sph_set_eos_ideal(self.h, k, float(d["gamma"])))
        else:
            raise ValueError(d["kind"])

    def eos_eval(self, k: int, quantity: str, a, b):
        """EoS_t quantity of material k on the device: (values, undefined count); a = rho, b = u
        (or s for internal_energy)"""
        a = np.ascontiguousarray(a, np.float64).reshape(-1)
        b = np.ascontiguousarray(b, np.float64).reshape(-1)
        assert a.shape == b.shape
        out = np.empty_like(a)
        undef = C.c_int64()
        self._check(self.L.sph_eos_eval(self.h, k, EOS_QUANTITY[quantity], len(a), _ptr(a), _ptr(b), _ptr(out),
                                        C.byref(undef)))
        return out, int(undef.value)

    def load_table_file(self, k: int, path: str):
        self._check(self.L.sph_load_eos_table_file(self.h, k, path.encode()))

    # state ----------------------------------------------------------------
    def upload(self, F: np.ndarray, ids=None, mats=None, time=0.0, init_smth=False, dt=0.0, forces_valid=False,
               inputs_only=False):
        """inputs_only: copy only STEP_INPUT_FIELDS (SPH_UPLOAD_STEP_INPUTS)"""
        F = np.ascontiguousarray(F, np.float64)
        assert F.shape[0] == NFIELD
        n = F.shape[1]
        ids = None if ids is None else np.ascontiguousarray(ids, np.int64)
        mats = None if mats is None else np.ascontiguousarray(mats, np.int32)
        flags = (1 if init_smth else 0) | (2 if forces_valid else 0) | (4 if inputs_only else 0)
        self._check(self.L.sph_upload(self.h, n, _ptr(F), F.shape[1], _ptr(ids), _ptr(mats), float(time), float(dt),
                                      flags))
        self.n = n

    def download(self, out: np.ndarray | None = None):
        if out is None:
            out = np.empty((NFIELD, self.n), np.float64)
        ids = np.empty(self.n, np.int64)
        mats = np.empty(self.n, np.int32)
        self._check(self.L.sph_download(self.h, _ptr(out), out.shape[1], _ptr(ids), _ptr(mats)))
        return out, ids, mats

    def download_fields(self, out: np.ndarray, names):
        """copies the named fields (e.g. STEP_OUTPUT_FIELDS) into the rows of `out` (field-major,
        upload order); the other rows are left as they are"""
        mask = 0
        for f in names:
            mask |= 1 << FIELD[f]
        assert out.shape[0] == NFIELD and out.flags["C_CONTIGUOUS"]
        self._check(self.L.sph_download_fields(self.h, _ptr(out), out.shape[1], mask, None, None))
        return out

    def step_download(self, out: np.ndarray, names):
        """one step whose named fields reach `out` (field-major, upload order) as soon as the step
        has written them (pin `out` for the copies to overlap the step)"""
        mask = 0
        for f in names:
            mask |= 1 << FIELD[f]
        assert out.shape[0] == NFIELD and out.flags["C_CONTIGUOUS"]
        self._check(self.L.sph_step_download(self.h, _ptr(out), out.shape[1], mask))
        return out

    def prologue(self):
        self._check(self.L.sph_prologue(self.h))

    # several runs in one context ------------------------------------------------
    def add_run(self, F: np.ndarray, ids=None, mats=None, time=0.0, init_smth=False, dt=0.0, forces_valid=False):
        """appends a run (advanced with the others from the next step on); returns its handle"""
        F = np.ascontiguousarray(F, np.float64)
        assert F.shape[0] == NFIELD
        ids = None if ids is None else np.ascontiguousarray(ids, np.int64)
        mats = None if mats is None else np.ascontiguousarray(mats, np.int32)
        flags = (1 if init_smth else 0) | (2 if forces_valid else 0)
        h = C.c_int64()
        self._check(self.L.sph_add_run(self.h, F.shape[1], _ptr(F), F.shape[1], _ptr(ids), _ptr(mats), float(time),
                                       float(dt), flags, C.byref(h)))
        self.n = self.n_particles()
        return h.value

    def remove_run(self, handle: int):
        self._check(self.L.sph_remove_run(self.h, int(handle)))
        self.n = self.n_particles()

    def runs(self):
        n = C.c_int()
        self._check(self.L.sph_list_runs(self.h, None, 0, C.byref(n)))
        hs = np.zeros(max(1, n.value), np.int64)
        self._check(self.L.sph_list_runs(self.h, _ptr(hs), len(hs), C.byref(n)))
        return hs[:n.value].tolist()

    def run_info(self, handle: int):
        n, t, dt, st = C.c_int64(), C.c_double(), C.c_double(), C.c_int64()
        self._check(self.L.sph_run_info(self.h, int(handle), C.byref(n), C.byref(t), C.byref(dt), C.byref(st)))
        return dict(n=n.value, time=t.value, dt=dt.value, steps=st.value)

    def n_particles(self):
        return sum(self.run_info(h)["n"] for h in self.runs())

    def download_run(self, handle: int):
        n = self.run_info(handle)["n"]
        out = np.empty((NFIELD, n), np.float64)
        ids = np.empty(n, np.int64)
        mats = np.empty(n, np.int32)
        self._check(self.L.sph_download_run(self.h, int(handle), _ptr(out), n, _ptr(ids), _ptr(mats)))
        return out, ids, mats

    def autotune(self):
        """times the derivative / hydro kernels with 1, 2, 4 threads per particle on the current state
        (after a step) and keeps the fastest; returns the choices and the times (microseconds)"""
        p = np.zeros(8, np.int64)
        self._check(self.L.sph_autotune(self.h, 0, _ptr(p)))
        return {"drvt_tpi": int(p[0]), "hydro_tpi": int(p[1]), "drvt_us": p[2:5].tolist(), "hydro_us": p[5:8].tolist()}

    def set_tune(self, drvt_tpi=1, hydro_tpi=1):
        p = np.zeros(8, np.int64)
        p[0], p[1] = drvt_tpi, hydro_tpi
        self._check(self.L.sph_autotune(self.h, 1, _ptr(p)))

    def run_diagnostics(self, handle: int):
        out = np.zeros(8)
        self._check(self.L.sph_run_diagnostics(self.h, int(handle), _ptr(out)))
        return out

    def step(self, n_steps=1):
        self._check(self.L.sph_step(self.h, int(n_steps)))

    def time(self):
        t, dt, st = C.c_double(), C.c_double(), C.c_int64()
        self._check(self.L.sph_get_time(self.h, C.byref(t), C.byref(dt), C.byref(st)))
        return t.value, dt.value, st.value

    def diagnostics(self):
        out = np.zeros(8)
        self._check(self.L.sph_diagnostics(self.h, _ptr(out)))
        return out

    # inspection -------------------------------------------------------------
    def run_pass(self, p: int):
        self._check(self.L.sph_run_pass(self.h, int(p)))

    def order(self):
        slot = np.empty(self.n, np.int32)
        keys = np.empty(self.n, np.uint64)
        self._check(self.L.sph_get_order(self.h, _ptr(slot), _ptr(keys)))
        return slot, keys

    def neighbors(self, mode: int, k: int):
        n = C.c_int64()
        buf = np.empty(4096, np.int32)
        self._check(self.L.sph_get_neighbors(self.h, mode, int(k), _ptr(buf), len(buf), C.byref(n)))
        if n.value > len(buf):
            buf = np.empty(n.value, np.int32)
            self._check(self.L.sph_get_neighbors(self.h, mode, int(k), _ptr(buf), len(buf), C.byref(n)))
        return buf[:n.value].copy()

    def tree(self):
        nc = C.c_int64()
        self._check(self.L.sph_get_tree(self.h, C.byref(nc), None, None, None, None, None))
        n = nc.value
        start, count, level, nch = (np.empty(n, np.int32) for _ in range(4))
        com = np.empty((n, 4), np.float64)
        self._check(self.L.sph_get_tree(self.h, C.byref(nc), _ptr(start), _ptr(count), _ptr(level), _ptr(nch),
                                        _ptr(com)))
        return dict(start=start, count=count, level=level, n_child=nch, com=com)

    def n_groups(self):
        ng = C.c_int64()
        self._check(self.L.sph_get_grav_list(self.h, -1, C.byref(ng), None, 0, None, None, None, 0, None, None,
                                             None))
        return ng.value

    def grav_list(self, g: int):
        ne, ns, ng = C.c_int64(), C.c_int64(), C.c_int64()
        gs, gcnt = np.zeros(1, np.int32), np.zeros(1, np.int32)
        self._check(self.L.sph_get_grav_list(self.h, g, C.byref(ng), None, 0, C.byref(ne), None, None, 0,
                                             C.byref(ns), _ptr(gs), _ptr(gcnt)))
        epj = np.empty(max(1, ne.value), np.int32)
        lev = np.empty(max(1, ns.value), np.int32)
        st = np.empty(max(1, ns.value), np.int32)
        self._check(self.L.sph_get_grav_list(self.h, g, C.byref(ng), _ptr(epj), len(epj), C.byref(ne), _ptr(lev),
                                             _ptr(st), len(st), C.byref(ns), _ptr(gs), _ptr(gcnt)))
        return dict(start=int(gs[0]), count=int(gcnt[0]), epj=epj[:ne.value].copy(), spj_level=lev[:ns.value].copy(),
                    spj_start=st[:ns.value].copy())

    def grav_lists(self):
        """every gravity list of the last FP64 gravity pass: group start / count (sorted indices), EPJ
        runs (offset, length, sorted particle indices) and SPJ runs (offset, length, cell indices)"""
        ng, te, ts = C.c_int64(), C.c_int64(), C.c_int64()
        self._check(self.L.sph_get_grav_lists(self.h, C.byref(ng), C.byref(te), C.byref(ts), None, None, None, None,
                                              None, None, None, None))
        g = ng.value
        out = {k: np.empty(g, np.int32) for k in ("start", "count", "epj_off", "epj_len", "spj_off", "spj_len")}
        out["epj"] = np.empty(max(1, te.value), np.int32)
        out["spj"] = np.empty(max(1, ts.value), np.int32)
        self._check(self.L.sph_get_grav_lists(self.h, C.byref(ng), C.byref(te), C.byref(ts), _ptr(out["start"]),
                                              _ptr(out["count"]), _ptr(out["epj_off"]), _ptr(out["epj_len"]),
                                              _ptr(out["epj"]), _ptr(out["spj_off"]), _ptr(out["spj_len"]),
                                              _ptr(out["spj"])))
        out["epj"] = out["epj"][:te.value]
        out["spj"] = out["spj"][:ts.value]
        return out

    def enable_timing(self, on=True):
        self._check(self.L.sph_get_timings(self.h, None, -1 if on else -2, None))

    def reset_timing(self):
        self._check(self.L.sph_get_timings(self.h, None, -3, None))

    def timings(self):
        """accumulated device ms per segment (SEGMENTS order)"""
        buf = np.zeros(32)
        n = C.c_int()
        self._check(self.L.sph_get_timings(self.h, _ptr(buf), 32, C.byref(n)))
        return dict(zip(SEGMENTS, buf[:n.value].tolist()))

    def step_timed(self, n_steps=1):
        ms = C.c_double()
        self._check(self.L.sph_step_timed(self.h, int(n_steps), C.byref(ms)))
        return ms.value

    def counters(self):
        out = np.zeros(16, np.int64)
        self._check(self.L.sph_get_counters(self.h, _ptr(out)))
        keys = ["launches", "pairs_gather", "pairs_sym", "pairs_grav", "cells", "groups", "epj", "spj",
                "walks_full", "walks_repair", "skin_violators", "units_walked", "units", "row_capacity",
                "superset_entries", "spilled_entries"]
        return dict(zip(keys, out.tolist()))


# ---------------------------------------------------------------------------
# functor-compatible batch calls (MultiWalk dispatch / retrieve)

_KINDS = {
    "dens": (T.EPI_DENS, T.EPJ_DENS, T.RES_DENS),
    "drvt": (T.EPI_DRVT, T.EPJ_DRVT, T.RES_DRVT),
    "hydro": (T.EPI_HYDRO, T.EPJ_HYDRO, T.RES_HYDRO),
    "grav": (T.EPI_GRAV, T.EPJ_GRAV, T.RES_GRAV),
}


def _ptr_array(arrs):
    a = (C.c_void_p * max(1, len(arrs)))()
    for k, x in enumerate(arrs):
        a[k] = x.ctypes.data if len(x) else None
    return a


def dispatch(kind: str, tag: int, epi_list, epj_list, spj_list=None):
    L = load()
    n_walk = len(epi_list)
    for e, (di, dj, _) in zip(epi_list, [_KINDS[kind]] * n_walk):
        assert e.dtype == di
    n_epi = (C.c_int * max(1, n_walk))(*[len(e) for e in epi_list])
    n_epj = (C.c_int * max(1, n_walk))(*[len(e) for e in epj_list])
    pe, pj = _ptr_array(epi_list), _ptr_array(epj_list)
    if kind == "grav":
        spj_list = spj_list if spj_list is not None else [np.zeros(0, T.SPJ_MONO)] * n_walk
        n_spj = (C.c_int * max(1, n_walk))(*[len(s) for s in spj_list])
        ps = _ptr_array(spj_list)
        rc = L.sph_dispatch_grav(tag, n_walk, pe, n_epi, pj, n_epj, ps, n_spj)
    else:
        rc = getattr(L, f"sph_dispatch_{kind}")(tag, n_walk, pe, n_epi, pj, n_epj)
    if rc != SPH_OK:
        raise SphError(rc, L.sph_batch_last_error().decode())
    return n_epi


def dispatch_index(kind: str, tag: int, epi_list, id_list, epj_all=None, id_spj_list=None, spj_all=None,
                   send=False):
    """the index form (sph_dispatch_index_*): walk w's j entries are epj_all[id_list[w]] (and, for
    gravity, spj_all[id_spj_list[w]]); send=True first copies epj_all (and spj_all) to the device,
    as the first call of a pass does.  Returns n_epi for retrieve()."""
    L = load()
    n_walk = len(epi_list)
    for e in epi_list:
        assert e.dtype == _KINDS[kind][0]
    ids = [np.ascontiguousarray(a, dtype=np.int32) for a in id_list]
    n_epi = (C.c_int * max(1, n_walk))(*[len(e) for e in epi_list])
    n_epj = (C.c_int * max(1, n_walk))(*[len(a) for a in ids])
    pe, pj = _ptr_array(epi_list), _ptr_array(ids)
    ea = epj_all if epj_all is not None else np.zeros(0, _KINDS[kind][1])
    assert ea.dtype == _KINDS[kind][1] and ea.flags.c_contiguous
    if kind == "grav":
        sids = [np.ascontiguousarray(a, dtype=np.int32) for a in (id_spj_list if id_spj_list is not None
                                                                    else [np.zeros(0, np.int32)] * n_walk)]
        sa = spj_all if spj_all is not None else np.zeros(0, T.SPJ_MONO)
        n_spj = (C.c_int * max(1, n_walk))(*[len(a) for a in sids])
        rc = L.sph_dispatch_index_grav(tag, n_walk, pe, n_epi, pj, n_epj, _ptr_array(sids), n_spj,
                                       ea.ctypes.data if len(ea) else None, len(ea),
                                       sa.ctypes.data if len(sa) else None, len(sa), int(send))
    else:
        rc = getattr(L, f"sph_dispatch_index_{kind}")(tag, n_walk, pe, n_epi, pj, n_epj,
                                                      ea.ctypes.data if len(ea) else None, len(ea), int(send))
    if rc != SPH_OK:
        raise SphError(rc, L.sph_batch_last_error().decode())
    return n_epi   # the call has read the index arrays: they may go


def retrieve(kind: str, tag: int, n_epi):
    L = load()
    res_dt = _KINDS[kind][2]
    n_walk = len(n_epi) if hasattr(n_epi, "__len__") else 0
    outs = [np.empty(n_epi[w], res_dt) for w in range(n_walk)]
    pr = _ptr_array(outs)
    rc = getattr(L, f"sph_retrieve_{kind}")(tag, n_walk, n_epi, pr)
    if rc != SPH_OK:
        raise SphError(rc, L.sph_batch_last_error().decode())
    return outs


def batch_precision(precision: str):
    """arithmetic of the batch entry points' next dispatches: "fp64" (the reference functors) or
    "mixed" (sph_batch_set_precision)"""
    if precision not in ("fp64", "mixed"):
        raise ValueError(f"precision must be 'fp64' or 'mixed', not {precision!r}")
    L = load()
    rc = L.sph_batch_set_precision(PREC_MIXED if precision == "mixed" else PREC_FP64)
    if rc != SPH_OK:
        raise SphError(rc, L.sph_batch_last_error().decode())


BATCH_STAGING = {"auto": 0, "host": 1, "device": 2}   # SPH_BATCH_STAGING_*


def batch_staging(mode: str):
    """who moves the next dispatches' walks to the device (sph_batch_set_staging): "auto" (the GPU
    gathers them from host memory where it can read pageable memory, else the host copies them),
    "host" or "device" """
    if mode not in BATCH_STAGING:
        raise ValueError(f"staging must be one of {sorted(BATCH_STAGING)}, not {mode!r}")
    L = load()
    rc = L.sph_batch_set_staging(BATCH_STAGING[mode])
    if rc != SPH_OK:
        raise SphError(rc, L.sph_batch_last_error().decode())


def run_walks(kind: str, epi_list, epj_list, spj_list=None, tag: int = 0):
    """dispatch + retrieve: the reference functor applied to each walk on the GPU."""
    n_epi = dispatch(kind, tag, epi_list, epj_list, spj_list)
    if len(epi_list) == 0:
        return []
    return retrieve(kind, tag, n_epi)


def probe_peak(fp64: bool, device: int = 0) -> float:
    """Measured FMA rate of the device, TFLOP/s."""
    L = load()
    t = C.c_double()
    rc = L.sph_probe_peak(device, 1 if fp64 else 0, C.byref(t))
    if rc != SPH_OK:
        raise SphError(rc, "sph_probe_peak failed")
    return t.value
