"""Build recipe for the CPU oracle (test infrastructure).

Compiles oracle/sph_oracle.c with gcc into two shared libraries under
oracle/_build/:

* ``liboracle.so``      -- IEEE build (``-ffp-contract=off``): the checker.
* ``liboracle_fast.so`` -- the reference's release flags
  (``-O3 -ffast-math -funroll-loops``, CMakeLists.txt:27-28) with OpenMP:
  the timed CPU baseline.

When the reference sources are present (this container, not the GPU host),
it also builds the reference leg ``oracle/_ref/ref_driver`` via
oracle/ref/Makefile.
"""
from __future__ import annotations

import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
BUILD = os.path.join(HERE, "_build")
# The reference checkout: $FDPS_SPH_REFERENCE, else a directory named "reference"
# beside this repository's root (absent on hosts that only run the prebuilt oracle).
REF_ROOT = os.environ.get("FDPS_SPH_REFERENCE") or os.path.normpath(os.path.join(HERE, "..", "..", "reference"))


def _cc(out: str, flags: list[str]) -> None:
    src = os.path.join(HERE, "sph_oracle.c")
    cmd = ["gcc", "-std=c11", "-shared", "-fPIC", "-fopenmp", *flags, src, "-o", out, "-lm"]
    subprocess.run(cmd, check=True)


def build(force: bool = False) -> None:
    os.makedirs(BUILD, exist_ok=True)
    src = os.path.join(HERE, "sph_oracle.c")
    hdr = os.path.join(HERE, "sph_oracle.h")
    newest = max(os.path.getmtime(src), os.path.getmtime(hdr), os.path.getmtime(__file__))
    targets = {
        "liboracle.so": ["-O2", "-ffp-contract=off", "-fno-fast-math"],
        "liboracle_fast.so": ["-O3", "-ffast-math", "-funroll-loops"],
    }
    for name, flags in targets.items():
        out = os.path.join(BUILD, name)
        if force or not os.path.exists(out) or os.path.getmtime(out) < newest:
            _cc(out, flags)
    if os.path.isdir(os.path.join(REF_ROOT, "src")):
        subprocess.run(["make", "-s", "-C", os.path.join(HERE, "ref"), f"REF_ROOT={REF_ROOT}"], check=True)


if __name__ == "__main__":
    build(force="--force" in sys.argv)
