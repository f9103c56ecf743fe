"""Snapshot text format (the reference's writeParticleAscii of RealPtcl) and
the pointer-free checkpoint; host only."""
import os

import numpy as np
import pytest

from fdps_sph_gb300 import ic, snapshot

from oracle import build_oracle

# the reference's initial state, when the reference checkout is present ($FDPS_SPH_REFERENCE, or beside this repo)
REF_SNAPSHOT = os.path.join(build_oracle.REF_ROOT, "input", "tar.dat")


def test_ascii_round_trip(tmp_path):
    F, ids, mats, _ = ic.config_small_impact(seed=3, n_target=300, n_impactor=40)
    path = snapshot.write_ascii(str(tmp_path / "results.00003"), F, ids, mats, 1234.5)
    assert path.endswith("results.00003_00001_00000.dat")
    G, gid, gtag, t = snapshot.read_ascii(path)
    assert t == float("%e" % 1234.5)
    assert np.array_equal(gid, ids) and np.array_equal(gtag, mats)
    for c in ("mass", "x", "y", "z", "vx", "vy", "vz", "dens", "eng", "pres", "pot"):
        k = ic.FIELD[c]
        want = np.array([float("%f" % v) for v in F[k]])
        assert np.array_equal(G[k], want), c
    with open(path) as fh:
        head = [fh.readline() for _ in range(3)]
    assert head[1].strip() == str(F.shape[1]) and len(head[2].split("\t")) == 15


@pytest.mark.skipif(not os.path.exists(REF_SNAPSHOT), reason="the reference's input snapshot is not present")
def test_reads_the_reference_snapshot():
    F, ids, tags, t = snapshot.read_ascii(REF_SNAPSHOT)
    assert F.shape[1] == 15000 and abs(t - 1.000777e4) < 1e-2
    assert np.array_equal(ids, np.arange(15000))
    f = ic.FIELD
    # densities at or above the FLAG_GI floor of 5 (force.h:18-20): the state holds isolated particles
    assert (F[f["mass"]] > 0).all() and (F[f["dens"]] >= 5.0).all() and (F[f["eng"]] > 0).all()
    assert (F[f["dens"]] == 5.0).any() and F[f["dens"]].max() > 3000
    assert set(np.unique(tags)) <= {0, 1}


class _FakeContext:
    """the three context calls write_checkpoint uses"""

    def __init__(self, runs):
        self._runs = runs

    def runs(self):
        return list(range(len(self._runs)))

    def run_info(self, h):
        return self._runs[h][3]

    def download_run(self, h):
        return self._runs[h][:3]


def test_checkpoint_round_trip(tmp_path):
    runs = []
    for k, (nt, ni) in enumerate(((200, 30), (120, 20))):
        F, ids, mats, _ = ic.config_small_impact(seed=10 + k, n_target=nt, n_impactor=ni)
        F[ic.FIELD["dt"]] = 1.5 + k
        runs.append((F, ids, mats, {"n": F.shape[1], "time": 10.0 * k + 0.25, "dt": 1.5 + k, "steps": 7 * k}))
    path = str(tmp_path / "run.ckpt")
    snapshot.write_checkpoint(path, _FakeContext(runs))
    back = snapshot.read_checkpoint(path)
    assert len(back) == 2
    for (F, ids, mats, info), (G, gid, gm, ginfo) in zip(runs, back):
        assert np.array_equal(F, G) and np.array_equal(ids, gid) and np.array_equal(mats, gm)
        assert ginfo == {"time": info["time"], "dt": info["dt"], "steps": info["steps"]}
    with open(path, "r+b") as fh:
        fh.write(b"NOTACKPT")
    with pytest.raises(ValueError):
        snapshot.read_checkpoint(path)
