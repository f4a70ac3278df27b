"""The ccf_gpu command line: the reference main_ccf's options, messages and
exit codes (src/main_ccf.cu), and an end-to-end run on the GPU."""
import os
import subprocess

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CLI = os.path.join(ROOT, "ccf_gb300", "lib", "ccf_gpu")


def run(*args):
    r = subprocess.run([CLI, *args], capture_output=True, text=True, timeout=300)
    return r.returncode, r.stdout, r.stderr


@pytest.mark.skipif(not os.path.exists(CLI), reason="ccf_gpu not built")
def test_help_and_argument_errors():
    rc, out, _ = run("-h")
    assert rc == 255 and "Usage:" in out and "--num_branches" in out
    rc, _, err = run("-k")
    assert rc == 255 and "Invalid input syntax" in err
    rc, _, err = run("-k", "0.3", "--bogus", "1")
    assert rc == 255 and "Unknown option --bogus" in err
    rc, _, err = run("-k", "abc")
    assert rc == 255 and "Invalid kappa_tot input" in err
    rc, _, err = run("-s", "1.5")
    assert rc == 255 and "smooth_fraction must be < 1" in err
    rc, _, err = run("-s", "-0.5")
    assert rc == 255 and "smooth_fraction must be >= 0" in err
    rc, _, err = run("-pr", "fp16")
    assert rc == 255 and "Invalid precision input" in err
    rc, _, err = run("-ct", "newton")
    assert rc == 255 and "Invalid continuation input" in err
    rc, out, _ = run("-h")
    assert "--continuation" in out


@pytest.mark.gpu
def test_cli_run_writes_the_reference_files(tmp_path):
    from oracle import oracle as O
    prefix = str(tmp_path) + "/"
    rc, out, err = run("-v", "0", "-k", "0.3", "-ks", "0.3", "-y", "0.1", "-t", "1", "-mf", "Equal", "-r", "0",
                       "-ns", "100", "-np", "100", "-nb", "1", "-rs", "1234", "-wls", "1", "-o", prefix)
    assert rc == 0, err
    for f in ("ccf_parameter_info.txt", "ccf_stars.bin", "ccf_ccs.bin", "ccf_caustics.bin", "ccf_mu_length_scales.bin"):
        assert os.path.exists(prefix + f), f
    ccs = O.read_array(prefix + "ccf_ccs.bin", is_complex=True)
    ref = O.run(num_threads=4, polish_tol=1e-13, polish_max_iters=80, kappa_tot=0.3, kappa_star=0.3, shear=0.1,
                num_stars=100, num_phi=100, num_branches=1, random_seed=1234)
    m = O.match_sets(ccs, ref["ccs"], 1)
    assert m["max_dist"] <= 1e-9 and m["non_bijective_cols"] == 0
    p = O.read_params(prefix + "ccf_parameter_info.txt")
    assert p["mass_function"] == "equal" and p["num_roots"] == 200
    # smooth fraction sets kappa_star = (1 - s) kappa_tot (src/main_ccf.cu:497-502)
    rc, _, err = run("-v", "0", "-k", "0.4", "-s", "0.25", "-ns", "50", "-np", "8", "-rs", "7", "-ws", "0", "-wcc", "0",
                     "-wc", "0", "-o", prefix + "s_")
    assert rc == 0, err
    p = O.read_params(prefix + "s_ccf_parameter_info.txt")
    assert abs(p["kappa_star"] - 0.3) < 1e-12
