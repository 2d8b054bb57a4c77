"""NumPy restatement of the spinful model's magnetic translation (test infrastructure).

BLQH_with_spin/basis.cpp:401-477: every nphi-bit block of a 4 * nphi-bit state
rotates by the same number of orbitals; the fermion sign counts, per block,
(electrons that do not wrap) x (electrons that wrap). Used by the CPU tests to
pin the orbit periods (basis_C) and representatives of the golden fixtures.
"""
from __future__ import annotations


def translate(c, bits, nphi, inverse=False):
    """(translated state, sign) of basis::translate / inv_translate."""
    mask = (1 << nphi) - 1
    msign = ((1 << bits) - 1) if inverse else (((1 << bits) - 1) << (nphi - bits))
    out, nsign = 0, 0
    for b in range(4):
        x = (c >> (b * nphi)) & mask
        ncross, nb = bin(x & msign).count("1"), bin(x).count("1")
        nsign += (nb - ncross) * ncross
        if inverse:
            y = ((x >> bits) | (x << (nphi - bits))) & mask
        else:
            y = ((x << bits) | (x >> (nphi - bits))) & mask
        out |= y << (b * nphi)
    return out, (-1 if nsign % 2 else 1)


def period(c, nphi):
    """basis_C: the smallest n in 1..nphi-1 with inv_translate(c, n) == c, else nphi (basis.cpp:129-135)."""
    for n in range(1, nphi):
        if translate(c, n, nphi, inverse=True)[0] == c:
            return n
    return nphi


def orbit(c, nphi):
    return {translate(c, n, nphi, inverse=True)[0] for n in range(nphi)}
