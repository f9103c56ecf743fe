"""The C++ host surface (include/fdps_sph_gb300.hpp) used the way the
reference's host code calls its functors: a program with class.h-shaped
payload types calls CalcDensity / CalcHydroForce / CalcGravityForce on golden
walks; results must match the reference functors' (tests/golden), also when
eight threads call the functors at once, and through the MultiWalk dispatch /
retrieve callbacks in payload and index form."""
import os
import struct
import subprocess

import numpy as np
import pytest

from fdps_sph_gb300 import build, ic, layouts as T
from helpers import load_golden, rel_err, vec_rel_err

pytestmark = pytest.mark.gpu
ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _walk(fun, key, w):
    s, c, jo, ji = (fun[key + "_walks_" + k] for k in ("start", "count", "joff", "jidx"))
    return int(s[w]), int(c[w]), ji[jo[w]:jo[w + 1]]


def test_cpp_functors_match_reference(tmp_path):
    lib = build.build()
    exe = str(tmp_path / "functor_host")
    subprocess.run(["g++", "-std=c++14", "-O2", "-pthread", "-I", os.path.join(ROOT, "include"),
                    os.path.join(ROOT, "tests", "cpp", "functor_host.cpp"), "-o", exe, "-L", os.path.dirname(lib),
                    "-lsph_gb300", f"-Wl,-rpath,{os.path.dirname(lib)}"], check=True)
    fun = load_golden("functors.npz")
    ids = fun["ids"]
    payload = []
    # density walk 0
    F = fun["state_dens"]
    s, n, js = _walk(fun, "dens", 0)
    a = np.zeros(n, T.EPI_DENS)
    a["pos"] = F[[0, 1, 2], s:s + n].T
    a["mass"] = F[ic.FIELD["mass"], s:s + n]
    a["smth"] = F[ic.FIELD["smth"], s:s + n]
    a["id"] = ids[s:s + n]
    b = np.zeros(len(js), T.EPJ_DENS)
    b["pos"] = F[[0, 1, 2]][:, js].T
    b["mass"] = F[ic.FIELD["mass"], js]
    b["smth"] = F[ic.FIELD["smth"], js]
    payload += [struct.pack("<i", n), a.tobytes(), struct.pack("<i", len(js)), b.tobytes()]
    dens_ref = fun["ref_dens"][s:s + n]
    # hydro walk 1 (superset)
    F = fun["state_hydro"]
    s2, n2, js2 = _walk(fun, "hydro", 1)
    a = np.zeros(n2, T.EPI_HYDRO)
    a["pos"] = F[[0, 1, 2], s2:s2 + n2].T
    a["vel"] = F[[3, 4, 5], s2:s2 + n2].T
    for k in ("smth", "dens", "pres", "snds", "grad_smth"):
        a[k] = F[ic.FIELD[k], s2:s2 + n2]
    a["Bal"] = F[ic.FIELD["bal"], s2:s2 + n2]
    a["AVa"] = F[ic.FIELD["ava"], s2:s2 + n2]
    b = np.zeros(len(js2), T.EPJ_HYDRO)
    b["pos"] = F[[0, 1, 2]][:, js2].T
    b["vel"] = F[[3, 4, 5]][:, js2].T
    for k in ("dens", "mass", "smth", "pres", "grad_smth", "snds"):
        b[k] = F[ic.FIELD[k], js2]
    b["Bal"] = F[ic.FIELD["bal"], js2]
    b["AVa"] = F[ic.FIELD["ava"], js2]
    payload += [struct.pack("<i", n2), a.tobytes(), struct.pack("<i", len(js2)), b.tobytes()]
    hyd_ref = fun["ref_hydro_superset"][s2:s2 + n2]
    # gravity walk 0
    s3, n3, js3 = _walk(fun, "grav", 0)
    a = np.zeros(n3, T.EPI_GRAV)
    a["pos"] = F[[0, 1, 2], s3:s3 + n3].T
    a["eps2"] = F[ic.FIELD["smth"], s3:s3 + n3] ** 2
    b = np.zeros(len(js3), T.EPJ_GRAV)
    b["pos"] = F[[0, 1, 2]][:, js3].T
    b["mass"] = F[ic.FIELD["mass"], js3]
    off = fun["grav_spj_off"]
    sp = np.ascontiguousarray(fun["grav_spj"][off[0]:off[1]])
    payload += [struct.pack("<i", n3), a.tobytes(), struct.pack("<i", len(js3)), b.tobytes(),
                struct.pack("<i", len(sp)), sp.tobytes()]
    grav_ref = fun["ref_grav"][s3:s3 + n3]
    fin, fout = tmp_path / "in.bin", tmp_path / "out.bin"
    fin.write_bytes(b"".join(payload))
    subprocess.run([exe, str(fin), str(fout)], check=True)
    raw = fout.read_bytes()
    o = 0
    d = np.frombuffer(raw[o:o + n * 16], T.RES_DENS)
    o += n * 16
    hres = np.frombuffer(raw[o:o + n2 * 40], T.RES_HYDRO)
    o += n2 * 40
    g = np.frombuffer(raw[o:o + n3 * 40], T.RES_GRAV)
    o += n3 * 40
    # eight threads calling the density and hydro functors concurrently (each on a tag of its own)
    # got the single-threaded results bit for bit
    assert np.frombuffer(raw[o:o + 4], np.int32)[0] == 0
    o += 4
    # the hydro walk through DispatchHydro / RetrieveHydro and through DispatchIndexHydro (send, then
    # the walk as indices): both bit-identical to the functor call (0: no flag raised)
    assert np.frombuffer(raw[o:o + 4], np.int32)[0] == 0
    assert rel_err(d["dens"], dens_ref["dens"], 1e-300) < 1e-12
    assert rel_err(d["smth"], dens_ref["smth"], 1e-300) < 1e-12
    assert vec_rel_err(hres["acc"], hyd_ref["acc"], 1e-6) < 1e-10
    assert rel_err(hres["dt"], hyd_ref["dt"], 1e-300) < 1e-13
    assert vec_rel_err(g["acc"], grav_ref["acc"], 1e-6) < 1e-11
    assert rel_err(g["pot"], grav_ref["pot"], 1e-300) < 1e-12
