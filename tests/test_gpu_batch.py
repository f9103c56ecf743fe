"""Functor-compatible batch entry points (sph_dispatch_* / sph_retrieve_*)
against the reference's own functors: the golden walks of
tests/golden/functors.npz (FDPS-style group supersets and exact lists) are
fed through the C ABI and compared with the reference outputs.

Tolerance: FP64 on both sides, differing only by fused multiply-adds and
the reference's -ffast-math reassociation: 1e-12 relative for positive sums
(density, h, potential, grad-h), 1e-10 normwise for sums with cancellation."""
import numpy as np
import pytest

from fdps_sph_gb300 import ic, layouts as T
from helpers import load_golden, rel_err, vec_rel_err

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def fun():
    return load_golden("functors.npz")


def walks(fun, key):
    s, c, jo, ji = (fun[key + "_walks_" + k] for k in ("start", "count", "joff", "jidx"))
    return [(int(s[w]), int(c[w]), ji[jo[w]:jo[w + 1]]) for w in range(len(s))]


def make(dt, F, ids, idx, fields):
    a = np.zeros(len(idx), dt)
    for name, src in fields.items():
        if name == "pos":
            a["pos"] = F[[0, 1, 2]][:, idx].T
        elif name == "vel":
            a["vel"] = F[[3, 4, 5]][:, idx].T
        elif name == "id":
            a["id"] = ids[idx]
        else:
            a[name] = F[ic.FIELD[src], idx]
    return a


def run(kind, fun, key, state, epi_fields, epj_fields, dt_i, dt_j, spj=None):
    from fdps_sph_gb300 import lib
    F = fun[state]
    ids = fun["ids"]
    W = walks(fun, key)
    epi = [make(dt_i, F, ids, np.arange(s, s + n), epi_fields) for s, n, _ in W]
    epj = [make(dt_j, F, ids, j, epj_fields) for _, _, j in W]
    out = lib.run_walks(kind, epi, epj, spj, tag=3)
    res = np.zeros(len(ids), out[0].dtype)
    for (s, n, _), o in zip(W, out):
        res[s:s + n] = o
    return res


DENS_I = {"pos": 0, "mass": "mass", "smth": "smth", "id": 0}
DENS_J = {"pos": 0, "mass": "mass", "smth": "smth"}
DRVT_I = {"pos": 0, "vel": 0, "smth": "smth", "dens": "dens"}
DRVT_J = {"pos": 0, "vel": 0, "mass": "mass", "smth": "smth"}
HYD_I = {"pos": 0, "vel": 0, "smth": "smth", "dens": "dens", "pres": "pres", "snds": "snds",
         "grad_smth": "grad_smth", "Bal": "bal", "AVa": "ava", "id": 0}
HYD_J = {"pos": 0, "vel": 0, "dens": "dens", "mass": "mass", "smth": "smth", "pres": "pres",
         "grad_smth": "grad_smth", "snds": "snds", "Bal": "bal", "AVa": "ava", "id": 0}


def test_batch_density(fun):
    r = run("dens", fun, "dens", "state_dens", DENS_I, DENS_J, T.EPI_DENS, T.EPJ_DENS)
    ref = fun["ref_dens"]
    assert rel_err(r["dens"], ref["dens"], 1e-300) < 1e-12
    assert rel_err(r["smth"], ref["smth"], 1e-300) < 1e-12


def test_batch_derivative(fun):
    r = run("drvt", fun, "drvt", "state_drvt", DRVT_I, DRVT_J, T.EPI_DRVT, T.EPJ_DRVT)
    ref = fun["ref_drvt"]
    assert rel_err(r["div_v"], ref["div_v"], 1e-9 * np.abs(ref["div_v"]).max()) < 1e-10
    assert vec_rel_err(r["rot_v"], ref["rot_v"], 1e-9) < 1e-10
    assert rel_err(r["grad_smth"], ref["grad_smth"], 1e-300) < 1e-12


@pytest.mark.parametrize("key,refkey", [("hydro", "ref_hydro_superset"), ("hydro_exact", "ref_hydro_exact")])
def test_batch_hydro(fun, key, refkey):
    r = run("hydro", fun, key, "state_hydro", HYD_I, HYD_J, T.EPI_HYDRO, T.EPJ_HYDRO)
    ref = fun[refkey]
    assert vec_rel_err(r["acc"], ref["acc"], 1e-6) < 1e-10
    assert rel_err(r["eng_dot"], ref["eng_dot"], 1e-6 * np.abs(ref["eng_dot"]).max()) < 1e-10
    # dt: v_sig_max over the walk's full list, superset semantics included
    assert rel_err(r["dt"], ref["dt"], 1e-300) < 1e-13


def test_batch_gravity(fun):
    spj_all, off = fun["grav_spj"], fun["grav_spj_off"]
    spj = [np.ascontiguousarray(spj_all[off[w]:off[w + 1]]) for w in range(len(off) - 1)]
    F = fun["state_hydro"]
    from fdps_sph_gb300 import lib
    ids = fun["ids"]
    W = walks(fun, "grav")
    epi = []
    for s, n, _ in W:
        a = np.zeros(n, T.EPI_GRAV)
        a["pos"] = F[[0, 1, 2]][:, s:s + n].T
        a["eps2"] = F[ic.FIELD["smth"], s:s + n] ** 2
        a["id"] = ids[s:s + n]
        epi.append(a)
    epj = [make(T.EPJ_GRAV, F, ids, j, {"pos": 0, "mass": "mass", "id": 0}) for _, _, j in W]
    out = lib.run_walks("grav", epi, epj, spj, tag=5)
    res = np.zeros(len(ids), T.RES_GRAV)
    for (s, n, _), o in zip(W, out):
        res[s:s + n] = o
    ref = fun["ref_grav"]
    assert vec_rel_err(res["acc"], ref["acc"], 1e-6) < 1e-11
    assert rel_err(res["pot"], ref["pot"], 1e-300) < 1e-12


def test_batch_empty_and_ragged_walks():
    from fdps_sph_gb300 import lib
    rng = np.random.default_rng(3)
    epi, epj = [], []
    for ni, nj in [(0, 5), (1, 0), (3, 1), (200, 300), (1, 1)]:
        a = np.zeros(ni, T.EPI_DENS)
        a["pos"] = rng.normal(size=(ni, 3))
        a["mass"] = 1.0
        a["smth"] = 0.7
        b = np.zeros(nj, T.EPJ_DENS)
        b["pos"] = rng.normal(size=(nj, 3))
        b["mass"] = 2.0
        b["smth"] = 0.7
        epi.append(a)
        epj.append(b)
    out = lib.run_walks("dens", epi, epj, tag=7)
    assert [len(o) for o in out] == [0, 1, 3, 200, 1]
    # an empty j-list gives the FLAG_GI floor (force.h:18-20)
    assert out[1]["dens"][0] == 5.0
    assert lib.run_walks("dens", [], [], tag=7) == []


def test_batch_mixed_precision_within_bar(fun):
    """sph_batch_set_precision(SPH_PREC_MIXED): the same golden walks, FP32 pair terms on
    walk-relative double-float coordinates, within the mixed path's 1e-5 of the reference functors
    (density and h relative per particle; vectors, du/dt and div v floored at the RMS); dt (a
    maximum of v_sig, no cancellation) to 1e-6.  The precision goes back to FP64 afterwards."""
    from fdps_sph_gb300 import lib
    from helpers import scalar_err_rms, vec_err_rms
    lib.batch_precision("mixed")
    try:
        d = run("dens", fun, "dens", "state_dens", DENS_I, DENS_J, T.EPI_DENS, T.EPJ_DENS)
        v = run("drvt", fun, "drvt", "state_drvt", DRVT_I, DRVT_J, T.EPI_DRVT, T.EPJ_DRVT)
        h = run("hydro", fun, "hydro", "state_hydro", HYD_I, HYD_J, T.EPI_HYDRO, T.EPJ_HYDRO)
    finally:
        lib.batch_precision("fp64")
    assert rel_err(d["dens"], fun["ref_dens"]["dens"], 1e-300) < 1e-5
    assert rel_err(d["smth"], fun["ref_dens"]["smth"], 1e-300) < 1e-5
    rv = fun["ref_drvt"]
    assert scalar_err_rms(v["div_v"], rv["div_v"]) < 1e-5
    assert vec_err_rms(v["rot_v"], rv["rot_v"]) < 1e-5
    assert rel_err(v["grad_smth"], rv["grad_smth"], 1e-300) < 1e-5
    rh = fun["ref_hydro_superset"]
    assert vec_err_rms(h["acc"], rh["acc"]) < 1e-5
    assert scalar_err_rms(h["eng_dot"], rh["eng_dot"]) < 1e-5
    assert rel_err(h["dt"], rh["dt"], 1e-300) < 1e-6


def _staging_supported(mode):
    """whether dispatches can run with this staging mode here (the device gather needs a GPU that
    reads pageable host memory)"""
    from fdps_sph_gb300 import lib
    lib.batch_staging(mode)
    try:
        a = np.zeros(1, T.EPI_DENS)
        a["smth"], a["mass"] = 1.0, 1.0
        b = np.zeros(1, T.EPJ_DENS)
        b["mass"], b["smth"] = 1.0, 1.0
        lib.run_walks("dens", [a], [b], tag=9)
        return True
    except lib.SphError as e:
        assert e.code == lib.SPH_ERR_STATE
        return False
    finally:
        lib.batch_staging("auto")


def test_batch_staging_modes_agree(fun):
    """the host copy and the device gather of the walks (sph_batch_set_staging) feed the kernels the
    same bytes, so every functor gives bit-identical results either way"""
    from fdps_sph_gb300 import lib
    if not _staging_supported("device"):
        pytest.skip("this GPU cannot read pageable host memory")
    out = {}
    for mode in ("host", "device"):
        lib.batch_staging(mode)
        try:
            out[mode] = (run("dens", fun, "dens", "state_dens", DENS_I, DENS_J, T.EPI_DENS, T.EPJ_DENS),
                         run("hydro", fun, "hydro", "state_hydro", HYD_I, HYD_J, T.EPI_HYDRO, T.EPJ_HYDRO))
        finally:
            lib.batch_staging("auto")
    for a, b in zip(out["host"], out["device"]):
        assert a.tobytes() == b.tobytes()


def test_batch_misaligned_walks_fall_back_to_the_host_copy():
    """a walk or RESULT array that is not 8-byte aligned cannot be moved in 8-byte words by the
    device: "auto" copies it on the host (same result as an aligned array), "device" refuses the
    dispatch"""
    from fdps_sph_gb300 import lib
    rng = np.random.default_rng(5)
    a = np.zeros(40, T.EPI_DENS)
    a["pos"] = rng.normal(size=(40, 3))
    a["mass"], a["smth"] = 1.0, 0.8
    b = np.zeros(60, T.EPJ_DENS)
    b["pos"] = rng.normal(size=(60, 3))
    b["mass"], b["smth"] = 1.5, 0.8
    raw = np.zeros(b.nbytes + 8, np.uint8)
    bm = np.frombuffer(raw.data, T.EPJ_DENS, count=len(b), offset=4)   # 4 bytes off alignment
    bm[:] = b
    assert bm.ctypes.data % 8 == 4
    ref = lib.run_walks("dens", [a], [b], tag=9)[0]
    got = lib.run_walks("dens", [a], [bm], tag=9)[0]
    assert got.tobytes() == ref.tobytes()
    # a RESULT array off alignment: the results come back through the host copy instead
    import ctypes as C
    n_epi = lib.dispatch("dens", 9, [a], [b])
    rraw = np.zeros(len(a) * T.RES_DENS.itemsize + 8, np.uint8)
    rm = np.frombuffer(rraw.data, T.RES_DENS, count=len(a), offset=4)
    assert rm.ctypes.data % 8 == 4
    rc = lib.load().sph_retrieve_dens(9, 1, n_epi, (C.c_void_p * 1)(rm.ctypes.data))
    assert rc == 0
    assert rm.tobytes() == ref.tobytes()
    if _staging_supported("device"):
        lib.batch_staging("device")
        try:
            with pytest.raises(lib.SphError) as e:
                lib.run_walks("dens", [a], [bm], tag=9)
            assert e.value.code == lib.SPH_ERR_STATE
        finally:
            lib.batch_staging("auto")


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_batch_index_form_equals_payload_form(fun, precision):
    """sph_dispatch_index_*: the pass's EPJ array sent once, the walks as indices into it -- the
    same j entries in the same order as the payload form, so bit-identical results"""
    from fdps_sph_gb300 import lib
    lib.batch_precision(precision)
    try:
        for kind, key, state, fi, fj, dti, dtj in [
                ("dens", "dens", "state_dens", DENS_I, DENS_J, T.EPI_DENS, T.EPJ_DENS),
                ("hydro", "hydro", "state_hydro", HYD_I, HYD_J, T.EPI_HYDRO, T.EPJ_HYDRO)]:
            F, ids = fun[state], fun["ids"]
            W = walks(fun, key)
            epi = [make(dti, F, ids, np.arange(s, s + n), fi) for s, n, _ in W]
            epj_all = make(dtj, F, ids, np.arange(len(ids)), fj)
            ref = lib.run_walks(kind, epi, [epj_all[j] for _, _, j in W], tag=3)
            n_epi = lib.dispatch_index(kind, 3, epi, [j for _, _, j in W], epj_all, send=True)
            got = lib.retrieve(kind, 3, n_epi)
            for a, b in zip(ref, got):
                assert a.tobytes() == b.tobytes(), kind
    finally:
        lib.batch_precision("fp64")


def test_batch_index_form_errors():
    """index walks before any send of their kind fail (SPH_ERR_STATE); an index outside the sent
    array fails the retrieve (SPH_ERR_ARG) without reading outside it"""
    from fdps_sph_gb300 import lib
    a = np.zeros(4, T.EPI_DRVT)
    a["smth"], a["dens"] = 1.0, 1.0
    b = np.zeros(6, T.EPJ_DRVT)
    b["mass"], b["smth"] = 1.0, 1.0
    b["pos"] = np.arange(18, dtype=float).reshape(6, 3) * 0.1
    # a fresh kind state cannot be guaranteed across tests, so the send of an empty array stands in
    lib.dispatch_index("drvt", 11, [], [], np.zeros(0, T.EPJ_DRVT), send=True)
    with pytest.raises(lib.SphError) as e:
        lib.dispatch_index("drvt", 11, [a], [np.arange(3)])
    assert e.value.code == lib.SPH_ERR_STATE
    n_epi = lib.dispatch_index("drvt", 11, [a], [np.array([0, 5, 6, 2])], b, send=True)   # 6 is outside
    with pytest.raises(lib.SphError) as e:
        lib.retrieve("drvt", 11, n_epi)
    assert e.value.code == lib.SPH_ERR_ARG
    n_epi = lib.dispatch_index("drvt", 11, [a], [np.array([0, 5, 1, 2])])   # the array is still there
    ok = lib.retrieve("drvt", 11, n_epi)[0]
    ref = lib.run_walks("drvt", [a], [b[[0, 5, 1, 2]]], tag=11)[0]
    assert ok.tobytes() == ref.tobytes()
