"""The allocation-free continuation entry point, ccf_continue_branch_noalloc.

It is meant for callers that cannot call cudaMalloc where they need more phi
steps of a branch -- a host framework that owns every byte of device memory
through its own pool, or a real-time loop that must not enter the
allocator.  Its row scratch lives in a fixed device array inside the
library instead.  This test gives it the branch-centre roots of a normal
ccf_run, lets it continue both sides of a branch, two calls in a row, and
checks every step it writes against the columns ccf_run produced for the same
branch and side with the full-sum continuation, which is the scheme the entry
point runs (same solver, so the tolerance of the parity tests, 1e-9
theta_star, is met with room to spare), in mixed precision and in FP64.
Between the first and the second call the device's free memory must not
change: the entry point allocates nothing (the first call may still load
code).  Device buffers come from torch, which is only plumbing here; the
entry point is called through the C ABI.

The file name makes pytest collect it after every other test.
"""
import ctypes

import numpy as np
import pytest

from ccf_gb300 import CCF, _lib

pytestmark = pytest.mark.gpu

CFG = dict(kappa_tot=0.45, kappa_star=0.35, shear=0.35, theta_star=1.0, mass_function="salpeter", m_lower=0.08,
           m_upper=1.5, m_solar=4.954984, rectangular=1, approx=1, num_stars=300, num_phi=64, num_branches=4,
           random_seed=4321)
TOL = 1e-9


@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_noalloc_continuation_matches_ccf_run(precision):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    c = CCF(**CFG)
    c.write_mu_length_scales = 0
    c.continuation = "aberth"
    c.precision = precision
    assert c.run(-1), c.last_error()
    ref = c.results(stars=False)
    info = ref["info"]
    R, nb = info["num_roots"], CFG["num_branches"]
    cols = CFG["num_phi"] // nb + 1
    half = CFG["num_phi"] // (2 * nb)
    L = _lib.load()
    dev = torch.device("cuda", 0)
    calls = [(1, 0), (1, 1)]
    bufs = []
    for branch, side in calls:   # every device buffer exists before the first call
        start = np.ascontiguousarray(ref["ccs"][branch::nb, half])          # centre roots of the branch
        bufs.append((torch.from_numpy(start.view(np.float64).copy()).to(dev),
                     torch.zeros(R * nb * cols * 2, dtype=torch.float64, device=dev),
                     torch.zeros(R * nb * cols, dtype=torch.float64, device=dev),
                     torch.zeros(R * nb * cols * 2, dtype=torch.float64, device=dev)))
    torch.cuda.synchronize()
    free_after = []
    for call, (branch, side) in enumerate(calls):
        start_d, ccs_d, errs_d, caus_d = bufs[call]
        rc = L.ccf_continue_branch_noalloc(c._h, branch, side, half, ctypes.c_void_p(start_d.data_ptr()),
                                           ctypes.c_void_p(ccs_d.data_ptr()), ctypes.c_void_p(errs_d.data_ptr()),
                                           ctypes.c_void_p(caus_d.data_ptr()), None)
        assert rc == 0, c.last_error()
        torch.cuda.synchronize()
        free_after.append(torch.cuda.mem_get_info(0)[0])
        got = ccs_d.cpu().numpy().view(np.complex128).reshape(R * nb, cols)
        got_w = caus_d.cpu().numpy().view(np.complex128).reshape(R * nb, cols)
        got_e = errs_d.cpu().numpy().reshape(R * nb, cols)
        steps = [half - j for j in range(1, half + 1)] if side == 0 else [half + j for j in range(1, half + 1)]
        for k in steps:
            np.testing.assert_allclose(got[branch::nb, k], ref["ccs"][branch::nb, k], rtol=0, atol=TOL)
            np.testing.assert_allclose(got_w[branch::nb, k], ref["caustics"][branch::nb, k], rtol=0, atol=TOL)
            # 1/mu errors: both within the 1e-9 target (the FP64 polish of ccf_run also
            # touched the centre roots this call starts from, so they may differ below it)
            np.testing.assert_allclose(got_e[branch::nb, k], ref["errs"][branch::nb, k], rtol=0, atol=TOL)
        # nothing outside the requested columns was written
        untouched = np.ones(cols, dtype=bool)
        untouched[steps] = False
        assert np.all(got[:, untouched] == 0)
        # every written 1/mu error is a plain non-negative number
        assert np.all(got_e[branch::nb, steps] >= 0)
    assert free_after[1] == free_after[0], "the second call changed the device's free memory"


def test_noalloc_rejects_bad_arguments():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("needs a GPU")
    L = _lib.load()
    c = CCF(**CFG)
    rc = L.ccf_continue_branch_noalloc(c._h, 0, 0, 1, None, None, None, None, None)
    assert rc == 6  # no field built yet
    assert c.run(-1), c.last_error()
    rc = L.ccf_continue_branch_noalloc(c._h, 9, 0, 1, None, None, None, None, None)
    assert rc == 1 and "branch" in c.last_error()
