"""GroupCutoff per molecule-kind pair (src/energy.h:740-768, src/energy.cpp:1868-1953).

The host helper turns the reference's input forms into the cutoff matrix (its
known-answer test, src/energy.cpp:1955-2002, with molecules M and Q); the
oracle's total energy with a per-pair matrix is checked against an independent
numpy sum over atom pairs whose groups' mass centres lie inside their pair's
cutoff; the descriptor rejects molecule ids outside the matrix.
"""
import dataclasses
import math

import numpy as np
import pytest

import faunus_gb300 as F
from faunus_gb300 import _capi as A
from faunus_gb300 import configs

import oracle_lib as O

MQ = ["M", "Q"]


def test_group_cutoff_json_forms_kat():
    # old style default
    assert np.array_equal(F.group_cutoff(12.0, MQ), np.full((2, 2), 12.0))
    # new style default
    assert np.array_equal(F.group_cutoff({"default": 13.0}, MQ), np.full((2, 2), 13.0))
    # custom: M-Q 14 in both orders (PairMatrix::set is symmetric), the rest the default
    c = F.group_cutoff({"default": 13.0, "M Q": 14.0}, MQ)
    assert c[0, 0] == 13.0 and c[0, 1] == c[1, 0] == 14.0 and c[1, 1] == 13.0
    # custom without a default: the other pairs have no cutoff
    c = F.group_cutoff({"M Q": 11.0}, MQ)
    assert math.isinf(c[0, 0]) and c[0, 1] == c[1, 0] == 11.0 and math.isinf(c[1, 1])


def _plain_water(cut, n_mol=64, L=15.0, seed=3):
    spec = configs.spce_water(n_mol=n_mol, L=L, cutoff_g2g=cut, molecules=tuple(MQ), seed=seed)
    return dataclasses.replace(spec, coulomb_type=A.FAU_COUL_PLAIN, coulomb_cutoff=0.0, ewald=None)


def _numpy_energy(spec, cut2):
    """Plain Coulomb + LJ over atom pairs of different molecules whose mass
    centres are closer than their kinds' cutoff (FP64, minimum image)."""
    x, L = spec.pos, spec.box
    gb = spec.group_begin
    g_of = np.repeat(np.arange(spec.n_groups), np.diff(gb))
    mol = spec.group_molid
    cm = spec.mass_center
    i, j = np.triu_indices(spec.n, 1)
    keep = g_of[i] != g_of[j]
    i, j = i[keep], j[keep]
    gi, gj = g_of[i], g_of[j]
    dcm = cm[gi] - cm[gj]
    dcm -= L * np.round(dcm / L)
    inside = (dcm * dcm).sum(1) < cut2[mol[gi], mol[gj]]
    i, j = i[inside], j[inside]
    d = x[i] - x[j]
    d -= L * np.round(d / L)
    r2 = (d * d).sum(1)
    ti, tj = spec.type[i], spec.type[j]
    s = spec.sigma2[ti, tj] / r2
    u = spec.bjerrum_length * spec.charge[i] * spec.charge[j] / np.sqrt(r2) + spec.eps4[ti, tj] * (s ** 6 - s ** 3)
    return float(u.sum()), len(i)


@pytest.mark.parametrize("cut", [{"default": 6.0, "M Q": 9.0}, {"M Q": 5.0}, 7.0])
def test_oracle_per_pair_cutoff_energy(cut):
    spec = _plain_water(cut)
    c = F.group_cutoff(cut, MQ)
    e_ref, n_pairs = _numpy_energy(spec, c * c)
    assert 0 < n_pairs < spec.n * (spec.n - 1) // 2  # some pairs are cut, some are not
    e = O.OracleSystem(spec).energy_total()["total"]
    assert abs(e - e_ref) <= 1e-10 * max(1.0, abs(e_ref))


def test_uniform_matrix_equals_scalar_cutoff():
    a = O.OracleSystem(_plain_water(7.0)).energy_total()["total"]
    b = O.OracleSystem(_plain_water({"default": 7.0})).energy_total()["total"]
    assert a == b


def test_descriptor_rejects_molid_outside_matrix():
    spec = _plain_water({"default": 6.0, "M Q": 9.0})
    bad = dataclasses.replace(spec, group_molid=np.where(np.arange(spec.n_groups) == 5, 2, spec.group_molid))
    with pytest.raises(F.FauError):
        F.footprint(bad)
    with pytest.raises(ValueError):
        dataclasses.replace(spec, cutoff_g2g_pairs=np.ones((2, 3))).to_desc()
