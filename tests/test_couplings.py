"""Coupling coefficients C and D (perturbations2.c:1236-1271).

The product computes them from closed forms of Clebsch-Gordan coefficients
(song2_host.c); the oracle from Wigner 3j symbols by the Racah formula.  The
special values quoted in the reference's comments pin the convention:
perturbations2.c:7897-7898, 7921-7922 (free-streaming terms of the dipole and
quadrupole equations).
"""
import math

import pytest


def prod(lib):
    return [lib.song2_coupling_c_minus, lib.song2_coupling_c_plus, lib.song2_coupling_d_minus,
            lib.song2_coupling_d_plus, lib.song2_coupling_d_zero]


def test_closed_forms_match_3j(lib, olib):
    fns = prod(lib)
    worst = 0.0
    for kind, f in enumerate(fns):
        for l in range(0, 45):
            for m in range(0, 5):
                if m > l:
                    continue
                for m1 in (m - 1, m, m + 1):
                    worst = max(worst, abs(f(l, m1, m) - olib.song2_oracle_coupling(kind, l, m1, m)))
    assert worst < 1e-12


@pytest.mark.parametrize("l,m1,m,val", [
    (1, 0, 0, 1.0),                      # dI(1,0) = k (I00 - 2/5 I20)
    (2, 0, 0, 2.0 / 3.0),                # dI(2,0) = k (2/3 I10 - 3/7 I30)
    (2, 1, 1, math.sqrt(3) / 3),         # dI(2,1) = k (sqrt3/3 I11 - sqrt8/7 I31)
    (1, 1, 1, 0.0),
])
def test_c_minus_reference_values(lib, l, m1, m, val):
    assert abs(lib.song2_coupling_c_minus(l, m1, m) - val) < 1e-15


@pytest.mark.parametrize("l,m1,m,val", [
    (1, 0, 0, 2.0 / 5.0),
    (1, 1, 1, math.sqrt(3) / 5),
    (2, 0, 0, 3.0 / 7.0),
    (2, 1, 1, math.sqrt(8) / 7),
])
def test_c_plus_reference_values(lib, l, m1, m, val):
    assert abs(lib.song2_coupling_c_plus(l, m1, m) - val) < 1e-15


def test_d_zero_vanishes_for_scalars(lib):
    # no scalar B-modes: d_zero(l,0,0) = 0 (perturbations2.c:6031-6039)
    for l in range(2, 40):
        assert lib.song2_coupling_d_zero(l, 0, 0) == 0.0
        assert abs(lib.song2_coupling_d_zero(l, 2, 2) - 4.0 / (l * (l + 1))) < 1e-15


def test_polarisation_starts_at_quadrupole(lib):
    for m in range(0, 3):
        assert lib.song2_coupling_d_minus(2, m, m) == 0.0
        assert lib.song2_coupling_d_plus(1, m, m) == 0.0
