"""The FDPS-style SPH j-lists of fdps_sph_gb300.walks hold every neighbour of every particle of
their group: gather (|x_j - x_i| < 2.5 h_i) and symmetric (< max(2.5 h_i, 2.5 h_j)), also for the
few particles with a smoothing length far above the rest (host only)."""
import numpy as np

from fdps_sph_gb300.walks import _sph_lists


def test_group_supersets_hold_every_neighbour():
    rng = np.random.default_rng(0)
    n = 3000
    pos = rng.random((n, 3))
    h = 0.02 * np.exp(rng.normal(0.0, 0.3, n))
    h[:5] *= 6.0   # a few isolated-particle-sized kernels
    o = np.argsort(pos[:, 0])
    pos, h = pos[o], h[o]
    start = np.arange(0, n, 100)
    count = np.full(len(start), 100)
    gi, go, si, so = _sph_lists(pos, h, start, count)
    for g, (s, c) in enumerate(zip(start, count)):
        G, S = set(gi[go[g]:go[g + 1]].tolist()), set(si[so[g]:so[g + 1]].tolist())
        assert np.all(np.diff(si[so[g]:so[g + 1]]) > 0)   # ascending, no repeats
        for i in range(s, s + c):
            d = np.linalg.norm(pos - pos[i], axis=1)
            assert set(np.flatnonzero(d < 2.5 * h[i]).tolist()) <= G
            assert set(np.flatnonzero(d < np.maximum(2.5 * h[i], 2.5 * h)).tolist()) <= S
