"""Known answer from the reference's equations: one star.

A star of mass m at z1 in a disc star field of radius rho (rectangular = 0),
with the approximate smooth mass, has kappa_star = m theta^2 / rho^2
(include/star.cuh:153-160) and alpha_smooth = -kappa_star z
(include/alpha_smooth.cuh:109-112, :225-228).  The critical-curve function
(include/ccf_functions.cuh:69-121, include/alpha_star.cuh:54-77) is then

    f(z) = gamma + theta^2 m / (z - z1)^2 - (1 - kappa + kappa_star) e^{-i phi},

so at every phi the two roots are z1 +- sqrt(theta^2 m / (A e^{-i phi} - gamma)),
A = 1 - kappa + kappa_star, and the caustic is
w = A z + gamma conj(z) - theta^2 m / conj(z - z1).  The oracle (the CPU
restatement of the reference) must find exactly these, to the reference's
stopping tolerance of 1e-9 theta_star."""
import numpy as np
import pytest

from oracle import oracle as O

CASES = [
    # m, z1, rho, theta, kappa, gamma, num_phi, num_branches
    (1.0, complex(0.3, -0.2), 5.0, 1.0, 0.3, 0.2, 16, 1),
    (0.5, complex(-1.0, 2.0), 8.0, 1.0, 0.6, 0.1, 24, 2),
    (2.0, complex(0.0, 0.5), 10.0, 1.0, 0.1, 0.5, 32, 4),
]


@pytest.mark.parametrize("m,z1,rho,theta,kappa,gamma,nphi,nb", CASES)
def test_one_star_roots_and_caustics(m, z1, rho, theta, kappa, gamma, nphi, nb):
    stars = {"stars": np.array([[z1.real, z1.imag, m]]), "rectangular": 0, "corner": complex(rho, 0),
             "theta_star": theta}
    r = O.run(stars=stars, num_threads=1, kappa_tot=kappa, shear=gamma, approx=1, num_phi=nphi,
              num_branches=nb, theta_star=theta)
    inf = r["info"]
    ks = m * theta ** 2 / rho ** 2
    assert inf["num_roots"] == 2
    assert inf["kappa_star_actual"] == pytest.approx(ks, rel=1e-14)

    # columns in the file layout: branch c, column k <-> phi = 2 pi (c nphi / nb + k) / nphi
    cols = nphi // nb + 1
    a = 1 - kappa + ks
    exp = np.zeros((2 * nb, cols), dtype=np.complex128)
    for c in range(nb):
        phi = 2 * np.pi * (c * nphi / nb + np.arange(cols)) / nphi
        s = np.sqrt(theta ** 2 * m / (a * np.exp(-1j * phi) - gamma))
        exp[0 * nb + c] = z1 + s      # row = root * num_branches + branch
        exp[1 * nb + c] = z1 - s
    match = O.match_sets(r["ccs"], exp, nb)
    assert match["non_finite"] == 0 and match["non_bijective_cols"] == 0
    assert match["max_dist"] <= 1e-9 * theta

    # the caustic is the lens map at the found root, in closed form
    z = r["ccs"]
    w = a * z + gamma * np.conj(z) - theta ** 2 * m / np.conj(z - z1)
    np.testing.assert_allclose(r["caustics"], w, rtol=1e-12, atol=1e-12 * theta)
    # and every point's 1/mu bound is below the reference's early-out level
    assert np.all(np.isfinite(r["errs"])) and r["errs"].max() < 1e-8
