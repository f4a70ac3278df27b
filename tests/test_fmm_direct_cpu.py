"""The tree + FMM deflection of the oracle against the direct sum over every
star, at random points of the field (a known answer from the reference's
equations: alpha = theta^2 sum m_i / conj(z - z_i) - kappa_star z for a disc
with the approximate smooth mass, include/alpha_star.cuh,
include/alpha_smooth.cuh:109-112).

The expansion order is chosen for alpha_error = 1e-7 theta_star
(include/ccf.cuh:439, :840-852).  With exact binomials the FMM meets it.  The
reference's int32 Pascal table (include/binomial_coefficients.cuh:41) wraps
above n = 33 while its M2L reads entries up to n = 2P - 1, which costs a few
1e-7 at P = 23: the oracle, like the library by default, keeps that table
for parity, and this test records the size of the effect."""
import numpy as np
import pytest

from oracle import oracle as O


def field(n, kappa_star, variable_mass, seed):
    rng = np.random.default_rng(seed)
    m = rng.uniform(0.1, 1.5, n) if variable_mass else np.ones(n)
    rho = np.sqrt(m.sum() / kappa_star)
    pos = rho * np.sqrt(rng.uniform(0, 1, n)) * np.exp(2j * np.pi * rng.uniform(0, 1, n))
    z = 0.95 * rho * np.sqrt(rng.uniform(0, 1, 2000)) * np.exp(2j * np.pi * rng.uniform(0, 1, 2000))
    stars = {"stars": np.stack([pos.real, pos.imag, m], 1), "rectangular": 0, "corner": complex(rho, 0),
             "theta_star": 1.0}
    direct = (m[None, :] / np.conj(z[:, None] - pos[None, :])).sum(1) - kappa_star * z
    return stars, z, direct


@pytest.mark.parametrize("n,kappa_star,variable_mass", [(300, 0.3, False), (1000, 0.5, True)])
def test_fmm_deflection_against_the_direct_sum(n, kappa_star, variable_mass):
    stars, z, direct = field(n, kappa_star, variable_mass, seed=7 + n)
    kw = dict(stars=stars, num_threads=2, kappa_tot=kappa_star + 0.1, shear=0.1, approx=1, num_phi=8,
              num_branches=1, theta_star=1.0)
    exact = O.eval_field(z, exact_binomials=1, **kw)
    assert exact["info"]["tree_levels"] >= 4
    err_exact = np.abs(exact["alpha"] - direct).max()
    assert err_exact <= 1e-7                      # the design error alpha_error
    wrapped = O.eval_field(z, exact_binomials=0, **kw)
    err_wrapped = np.abs(wrapped["alpha"] - direct).max()
    assert err_wrapped > 10 * err_exact           # the reference's table costs accuracy ...
    assert err_wrapped <= 1e-5                    # ... but stays a few 1e-7
