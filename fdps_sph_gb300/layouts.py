"""numpy mirrors of the reference's interaction payloads (src/class.h).

These are the byte layouts the C ABI's functor-compatible entry points take
(include/sph_gb300.h, ``sph_epi_dens`` etc.): every member is F64 or S64,
``PS::F64vec`` is three consecutive F64.
"""
from __future__ import annotations

import numpy as np

V3 = (np.float64, (3,))

# class.h:233-258
EPI_DENS = np.dtype([("pos", V3), ("mass", "f8"), ("smth", "f8"), ("id", "i8")])
# class.h:342-365
EPJ_DENS = np.dtype([("mass", "f8"), ("pos", V3), ("smth", "f8")])
# class.h:36-44
RES_DENS = np.dtype([("dens", "f8"), ("smth", "f8")])

# class.h:260-281
EPI_DRVT = np.dtype([("pos", V3), ("vel", V3), ("smth", "f8"), ("dens", "f8")])
# class.h:367-392
EPJ_DRVT = np.dtype([("mass", "f8"), ("pos", V3), ("vel", V3), ("smth", "f8")])
# class.h:47-58
RES_DRVT = np.dtype([("div_v", "f8"), ("rot_v", V3), ("grad_smth", "f8")])

# class.h:283-315
EPI_HYDRO = np.dtype([("pos", V3), ("vel", V3), ("smth", "f8"), ("dens", "f8"), ("pres", "f8"), ("snds", "f8"),
                      ("grad_smth", "f8"), ("Bal", "f8"), ("AVa", "f8"), ("id", "i8")])
# class.h:394-432
EPJ_HYDRO = np.dtype([("pos", V3), ("vel", V3), ("dens", "f8"), ("mass", "f8"), ("smth", "f8"), ("pres", "f8"),
                      ("grad_smth", "f8"), ("snds", "f8"), ("Bal", "f8"), ("AVa", "f8"), ("id", "i8")])
# class.h:61-72
RES_HYDRO = np.dtype([("acc", V3), ("eng_dot", "f8"), ("dt", "f8")])

# class.h:317-338
EPI_GRAV = np.dtype([("pos", V3), ("eps2", "f8"), ("id", "i8")])
# class.h:434-453
EPJ_GRAV = np.dtype([("pos", V3), ("mass", "f8"), ("id", "i8")])
# FDPS SPJMonopole (total mass, centre of mass)
SPJ_MONO = np.dtype([("mass", "f8"), ("pos", V3)])
# class.h:75-86
RES_GRAV = np.dtype([("acc", V3), ("pot", "f8"), ("dt", "f8")])

SIZES = {
    "epi_dens": 48, "epj_dens": 40, "res_dens": 16,
    "epi_drvt": 64, "epj_drvt": 64, "res_drvt": 40,
    "epi_hydro": 112, "epj_hydro": 120, "res_hydro": 40,
    "epi_grav": 40, "epj_grav": 40, "spj_mono": 32, "res_grav": 40,
}

for _name, _dt in [("epi_dens", EPI_DENS), ("epj_dens", EPJ_DENS), ("res_dens", RES_DENS),
                   ("epi_drvt", EPI_DRVT), ("epj_drvt", EPJ_DRVT), ("res_drvt", RES_DRVT),
                   ("epi_hydro", EPI_HYDRO), ("epj_hydro", EPJ_HYDRO), ("res_hydro", RES_HYDRO),
                   ("epi_grav", EPI_GRAV), ("epj_grav", EPJ_GRAV), ("spj_mono", SPJ_MONO), ("res_grav", RES_GRAV)]:
    assert _dt.itemsize == SIZES[_name], (_name, _dt.itemsize)


def result_clear(kind: str, n: int) -> np.ndarray:
    """RESULT::clear() (class.h:41-43, 53-57, 67-71, 81-85)."""
    dt = {"dens": RES_DENS, "drvt": RES_DRVT, "hydro": RES_HYDRO, "grav": RES_GRAV}[kind]
    r = np.zeros(n, dtype=dt)
    if kind in ("hydro", "grav"):
        r["dt"] = 1.0e30
    return r
