"""The reference's built-in geometry self-checks (perturbations2.c:5864-6065)
hold for every triplet of the oracle's geometrical corner: k1 sin(theta1) =
k2 sin(theta2), kz1 + kz2 = k, kx1 = -kx2, the l=1 rotation coefficients equal the
spherical components of k1, k2, k1.k2 is coordinate independent, rot(0,0) = 1,
c_minus_12(0,0) = 0, c_minus_12(1,0) = rot1*rot2, d_zero_12(l,0) = 0 and
X[m]^ij k_i k_j = c_minus(2,m) k k."""
import ctypes as C

from helpers import problem


def test_geometry_self_checks(lib, olib):
    p = problem(k_min=1e-4, k_max=0.3, k_size=7, k3_size=6, l_max=6, m=(0, 1, 2, 3, 4))
    dev = C.c_double()
    failures = []
    for (i1, i2, i3) in p.work_order():
        f = olib.song2_oracle_geometry_checks(C.byref(p.spec), i1, i2, i3, C.byref(dev))
        if f:
            failures.append((i1, i2, i3, f, dev.value))
    assert not failures, failures[:5]
