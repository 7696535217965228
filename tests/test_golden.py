"""The oracle reproduces its committed golden fixtures (tests/golden/*.npz,
made by tests/golden/make_golden.py)."""
import os

import numpy as np
import pytest

import oracle
from helpers import problem

HERE = os.path.dirname(os.path.abspath(__file__))
import sys  # noqa: E402
sys.path.insert(0, os.path.join(HERE, "golden"))
from make_golden import CASES  # noqa: E402


@pytest.mark.parametrize("name", sorted(CASES))
def test_oracle_matches_golden(lib, olib, name):
    g = np.load(os.path.join(HERE, "golden", name + ".npz"))
    p = problem(**CASES[name])
    fo = oracle.first_order(p, nthreads=4)
    assert np.allclose(fo, g["fo"], rtol=1e-9, atol=1e-12 * np.abs(g["fo"]).max())
    p.set_first_order(g["fo"])
    src, st = oracle.evolve(p, nthreads=4)
    assert np.array_equal(st["n_steps"], g["n_steps"])
    assert np.allclose(src, g["sources"], rtol=1e-9, atol=1e-12 * np.abs(g["sources"]).max())
