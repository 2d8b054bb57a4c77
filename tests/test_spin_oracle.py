"""Spinful golden fixtures (tests/golden/spin/, generated by the reference itself)
against the NumPy restatement of the four-block translation: orbit periods,
one representative per orbit, spin and layer counts. CPU only."""
import os

import numpy as np
import pytest

from conftest import ROOT
from oracle import spin_ref as S

SPIN = os.path.join(ROOT, "tests", "golden", "spin")
NAMES = sorted(f[:-4] for f in os.listdir(SPIN) if f.endswith(".npz"))


def load(name):
    return dict(np.load(os.path.join(SPIN, name + ".npz")))


@pytest.mark.parametrize("name", NAMES)
def test_periods_and_orbits(name):
    g = load(name)
    nphi, nel, nel_up, nel_su, J, K = (int(v) for v in g["spec"][:6])
    ids = [int(c) for c in g["id"]]
    assert ids == sorted(ids)
    assert [S.period(c, nphi) for c in ids] == [int(p) for p in g["period"]]
    if K >= 0:
        seen = set()
        for c in ids:
            o = frozenset(S.orbit(c, nphi))
            assert o not in seen  # one representative per orbit
            seen.add(o)
    m = (1 << nphi) - 1
    for c in ids:
        blk = [bin((c >> (b * nphi)) & m).count("1") for b in range(4)]
        assert sum(blk) == nel
        if nel_up >= 0:
            assert blk[0] + blk[1] == nel_up
        if nel_su >= 0:
            assert blk[0] + blk[2] == nel_su
        if J >= 0:
            assert sum(i % nphi for i in range(4 * nphi) if (c >> i) & 1) % nphi == J


def test_translation_is_a_group_action():
    nphi = 6
    rng = np.random.default_rng(0)
    for _ in range(200):
        c = int(rng.integers(0, 1 << (4 * nphi)))
        for n in range(1, nphi):
            t, s1 = S.translate(c, n, nphi)
            back, s2 = S.translate(t, n, nphi, inverse=True)
            assert back == c and s1 == s2
