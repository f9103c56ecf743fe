"""The reference's own EoS tables (eos/granite.rho_u.txt, eos/iron___.rho_u.txt) read by the
library's table reader and looked up, against the reference's classes reading the same files.

The library's reader (sph_read_eos_table_file, the one sph_load_eos_table_file uses; host only)
must give the arrays the reference's table constructor builds (EoS.h:121-221: density axis from
column 0 of each block's first line, energy axis from column 1 of the first block, pressure and
sound speed from columns 3 and 4), and the bilinear lookup on those arrays must give the
reference's Pressure / SoundSpeed (EoS.h:241-247, 394-400, interpolation.h:33-102).  The lookups
are evaluated by the oracle's restatement, which the golden tests pin to the same reference
classes; the device lookup is held to the oracle by the GPU EoS tests.  Needs the reference
checkout and the reference leg of the oracle (oracle/_ref), both of which exist only where the
reference sources are present: skipped elsewhere."""
import ctypes as C
import os
import struct
import subprocess
import tempfile

import numpy as np
import pytest

from oracle import build_oracle

REF = build_oracle.REF_ROOT
DRIVER = os.path.join(os.path.dirname(build_oracle.HERE), "oracle", "_ref", "ref_driver")
TABLES = ("eos/granite.rho_u.txt", "eos/iron___.rho_u.txt")

pytestmark = pytest.mark.skipif(not (os.path.exists(os.path.join(REF, TABLES[0])) and os.path.exists(DRIVER)),
                                reason="the reference checkout or its oracle leg is not present")


def _reference_lookups(path, pts):
    """(P, c_s) of the reference's ANEOS class reading `path`, at pts [n, 2] (rho, u)"""
    pb = path.encode()
    payload = (struct.pack("<i", len(pb)) + pb + struct.pack("<ii", 0, len(pts)) +
               np.ascontiguousarray(pts, dtype="<f8").tobytes())
    with tempfile.TemporaryDirectory() as td:
        fi, fo = os.path.join(td, "in.bin"), os.path.join(td, "out.bin")
        with open(fi, "wb") as fh:
            fh.write(payload)
        subprocess.run([DRIVER, "eos_file", fi, fo], check=True, cwd=REF)
        return np.fromfile(fo, dtype="<f8").reshape(-1, 2)


def _points(rng, rho, u, n=800):
    lr = np.log(rho[0]), np.log(rho[-1])
    lu = np.log(u[0]), np.log(u[-1])
    inner = np.stack([np.exp(rng.uniform(*lr, n)), np.exp(rng.uniform(*lu, n))], 1)
    ii, jj = rng.integers(0, len(rho), 50), rng.integers(0, len(u), 50)
    nodes = np.stack([rho[ii], u[jj]], 1)
    edges = np.array([[rho[0] * 0.5, u[5]], [rho[-1] * 2.0, u[5]], [rho[5], u[0] * 0.5], [rho[5], u[-1] * 2.0]])
    return np.concatenate([inner, nodes, edges])


@pytest.mark.parametrize("name", TABLES)
def test_reference_table_read_and_looked_up_as_the_reference_does(name):
    from fdps_sph_gb300 import eos, lib
    from oracle import pyoracle as po
    path = os.path.join(REF, name)
    rho, u, cols, ncols = lib.read_table_file(path)
    assert ncols == 6 and len(rho) == 120 and len(u) == 120
    # the product's Python reader gives the same arrays
    t = eos.read_rho_u(path)
    assert np.array_equal(t.rho, rho) and np.array_equal(t.u, u)
    assert np.array_equal(t.pres.reshape(-1), cols[3]) and np.array_equal(t.snds.reshape(-1), cols[4])
    assert np.array_equal(t.line_rho, cols[0]) and np.array_equal(t.line_u, cols[1])
    pts = _points(np.random.default_rng(7), rho, u)
    want = _reference_lookups(name, pts)
    L = po.lib()
    pres = np.ascontiguousarray(cols[3])
    snds = np.ascontiguousarray(cols[4])
    got = np.array([[L.or_table_lookup(po._p(rho), len(rho), po._p(u), len(u), po._p(pres), r, v),
                     L.or_table_lookup(po._p(rho), len(rho), po._p(u), len(u), po._p(snds), r, v)] for r, v in pts])
    scale = np.maximum(np.abs(want), 1e-300)
    assert np.max(np.abs(got - want) / scale) < 1e-13, float(np.max(np.abs(got - want) / scale))
