"""Device analysis, host side: the oracle's AtomRDF histogram (src/analysis.cpp:1556-1600,
bin floor(r / dr) of src/aux/equidistant_table.h:32-39) against a numpy restatement,
and the g(r) normalisation of PairFunction::_to_disk (src/analysis.cpp:724-737)."""
import math

import numpy as np

from faunus_gb300.system import rdf_normalise

import oracle_lib as O


def _np_hist(pos, types, L, ta, tb, dr, nb):
    i, j = np.triu_indices(len(pos), 1) if ta == tb else np.nonzero(np.ones((len(pos), len(pos)), bool))
    sel = (types[i] == ta) & (types[j] == tb)
    if ta == tb:
        sel &= i < j
    i, j = i[sel], j[sel]
    d = pos[i] - pos[j]
    d = np.where(d > L / 2, d - L, np.where(d < -L / 2, d + L, d))  # Cuboid::vdist
    r = np.sqrt(d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1] + d[:, 2] * d[:, 2])
    b = np.floor(r * (1.0 / dr)).astype(np.int64)
    h = np.bincount(np.minimum(b, nb), minlength=nb + 1)
    return h[:nb], int(h[nb])


def test_oracle_rdf_histogram_matches_numpy():
    rng = np.random.default_rng(5)
    L = np.array([20.0, 25.0, 30.0])
    pos = (rng.random((300, 3)) - 0.5) * L
    types = rng.integers(0, 3, 300).astype(np.int32)
    for ta, tb, dr, nb in ((0, 0, 0.1, 120), (0, 2, 0.25, 40), (1, 1, 0.05, 400)):
        h_o, beyond_o = O.rdf_hist(pos, types, L, ta, tb, dr, nb)
        h_n, beyond_n = _np_hist(pos, types, L, ta, tb, dr, nb)
        assert np.array_equal(h_o, h_n) and beyond_o == beyond_n
        n_a, n_b = (types == ta).sum(), (types == tb).sum()
        assert h_o.sum() + beyond_o == (n_a * (n_a - 1) // 2 if ta == tb else n_a * n_b)


def test_rdf_normalisation():
    dr, V = 0.5, 1000.0
    hist = np.array([0, 3, 5, 8, 0, 2], dtype=np.uint64)
    r, g = rdf_normalise(hist, dr, V)
    assert np.allclose(r, [0.5, 1.0, 1.5, 2.0, 2.5])
    tot = 18.0
    want = [hist[k] * V / (4 * math.pi * (k * dr) ** 2 * dr * tot) for k in range(1, 6)]
    assert np.allclose(g, want, rtol=1e-15)
