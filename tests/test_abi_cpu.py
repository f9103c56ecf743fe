"""CPU-side checks of the drop-in boundary: the library builds for sm_103a,
loads, and exports every entry point include/sph_gb300.h declares.  No
compute call is made (there is no GPU here)."""
import os
import re

import numpy as np

from fdps_sph_gb300 import build, lib, layouts as T

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_functions():
    src = open(os.path.join(ROOT, "include", "sph_gb300.h")).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    names = re.findall(r"\b(?:int|void|const char \*)\s*\*?\s*(sph_[a-z0-9_]+)\s*\(", src)
    return sorted(set(names))


def test_library_builds_and_exports_every_declared_symbol():
    path = build.build()
    assert os.path.exists(path)
    L = lib.load()
    names = declared_functions()
    assert len(names) >= 25
    for n in names:
        assert hasattr(L, n), f"missing export {n}"
    assert sorted(lib.EXPORTS) == names


def test_payload_layouts_match_header():
    # sizes in the header comments (class.h layouts) match the numpy mirrors
    src = open(os.path.join(ROOT, "include", "sph_gb300.h")).read()
    for name, size in T.SIZES.items():
        kind, _, part = name.partition("_")
        assert size % 8 == 0
    assert T.EPI_HYDRO.itemsize == 112 and T.EPJ_HYDRO.itemsize == 120
    assert "112 B" in src and "120 B" in src


def test_field_order_matches_header():
    src = open(os.path.join(ROOT, "include", "sph_gb300.h")).read()
    body = src[src.index("enum sph_field"):]
    body = body[:body.index("}")]
    names = re.findall(r"SPH_([A-Z]+)", body)
    names = [n for n in names if n != "NFIELD"]
    assert len(names) == lib.NFIELD
    from oracle import pyoracle as po
    assert po.FIELDS == lib.FIELDS
    assert np.all(np.array(names) == np.array([
        "X", "Y", "Z", "VX", "VY", "VZ", "MASS", "SMTH", "DENS", "ENG", "PRES", "SNDS", "DIVV", "ROTX", "ROTY",
        "ROTZ", "BAL", "AVA", "GRADH", "AX", "AY", "AZ", "ENGDOT", "VHX", "VHY", "VHZ", "ENGHALF", "DT", "GX",
        "GY", "GZ", "POT", "ENT", "TEMP"]))


def test_context_creation_fails_cleanly_without_gpu():
    import torch
    if torch.cuda.is_available():
        return
    try:
        lib.Context()
    except lib.SphError as e:
        assert e.code in (-2, -3)
    else:
        raise AssertionError("expected an error without a GPU")


def test_header_constants_match_binding():
    # every #define the Python binding mirrors as a number equals the header's
    src = open(os.path.join(ROOT, "include", "sph_gb300.h")).read()
    defs = {m.group(1): m.group(2) for m in re.finditer(r"#define\s+(SPH_[A-Z0-9_]+)\s+\(?(-?\d+)\)?", src)}
    assert int(defs["SPH_NOALLOC_MAX_N"]) == lib.NOALLOC_MAX_N
    assert int(defs["SPH_PREC_FP64"]) == lib.PREC_FP64 and int(defs["SPH_PREC_MIXED"]) == lib.PREC_MIXED
    assert int(defs["SPH_ERR_ARG"]) == lib.SPH_ERR_ARG and int(defs["SPH_ERR_STATE"]) == lib.SPH_ERR_STATE
    for mode, v in lib.BATCH_STAGING.items():
        assert int(defs["SPH_BATCH_STAGING_" + mode.upper()]) == v
    assert int(defs["SPH_ENTROPY_ABS_INT"]) == lib.ENTROPY_ABS_INT
    assert int(defs["SPH_ENTROPY_ABS_REAL"]) == lib.ENTROPY_ABS_REAL
    for code, name in lib.ERRORS.items():
        assert int(defs[name]) == code, name


def test_cpp_host_surface_compiles():
    # the C++ surface (include/fdps_sph_gb300.hpp: functors, MultiWalk payload and index callbacks)
    # instantiated with class.h-shaped payload types, as the GPU test's host program uses it
    import shutil
    import subprocess
    gxx = shutil.which("g++")
    if gxx is None:
        import pytest
        pytest.skip("no g++")
    subprocess.run([gxx, "-std=c++14", "-fsyntax-only", "-Wall", "-Werror=return-type", "-I",
                    os.path.join(ROOT, "include"), os.path.join(ROOT, "tests", "cpp", "functor_host.cpp")],
                   check=True)
