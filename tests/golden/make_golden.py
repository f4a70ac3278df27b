"""Generate the golden fixtures in this folder from the reference's own code.

The reference (weisluke/ccf) ships no tests or golden vectors, so its own FP64
functions are compiled for the host (``make -C oracle ref`` builds
``oracle/_ref/ccf_ref_host`` from the reference sources where they lie) and
run on small seeded fields.  Each case is stored as one compressed .npz with
the input parameters, the generated and tree-sorted star fields, the derived
parameters and the four output arrays in the reference's file layout.

Run from the repository root:  python tests/golden/make_golden.py
"""
from __future__ import annotations

import json
import os
import subprocess
import sys
import tempfile

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
from oracle import oracle as O  # noqa: E402

OPTS = {"kappa_tot": "-k", "kappa_star": "-ks", "shear": "-y", "theta_star": "-t", "mass_function": "-mf",
        "m_lower": "-ml", "m_upper": "-mh", "m_solar": "-ms", "rectangular": "-r", "approx": "-a",
        "num_stars": "-ns", "num_phi": "-np", "num_branches": "-nb", "random_seed": "-rs", "safety_scale": "-ss"}

CASES = {
    # the small plain-FP64 configuration: 100 equal masses in a disc, no smooth mass
    "disc_equal_n100": dict(kappa_tot=0.3, kappa_star=0.3, shear=0.1, theta_star=1, mass_function="equal",
                            rectangular=0, approx=1, num_stars=100, num_phi=100, num_branches=1, random_seed=1234),
    # rectangular field with smooth mass (Taylor alpha_smooth), Salpeter masses scaled to mean 1
    "rect_salpeter_n60": dict(kappa_tot=0.45, kappa_star=0.35, shear=0.35, theta_star=1, mass_function="salpeter",
                              m_lower=0.08, m_upper=1.5, m_solar=4.954984, rectangular=1, approx=1, num_stars=60,
                              num_phi=32, num_branches=4, random_seed=1235),
    # rectangular field, Kroupa broken power law
    "rect_kroupa_n50": dict(kappa_tot=0.7, kappa_star=0.6, shear=0.2, theta_star=1, mass_function="kroupa",
                            m_lower=0.08, m_upper=1.5, m_solar=1, rectangular=1, approx=1, num_stars=50,
                            num_phi=24, num_branches=2, random_seed=1236),
    # rectangular field with the exact (logarithmic) smooth-mass deflection
    "rect_exact_uniform_n40": dict(kappa_tot=0.5, kappa_star=0.4, shear=0.25, theta_star=1.3,
                                   mass_function="uniform", m_lower=0.1, m_upper=2, m_solar=1, rectangular=1,
                                   approx=0, num_stars=40, num_phi=16, num_branches=2, random_seed=77),
    # disc with the exact smooth-mass deflection, two-mass population
    "disc_exact_optdepth_n45": dict(kappa_tot=0.4, kappa_star=0.4, shear=0.3, theta_star=0.7,
                                    mass_function="optical_depth", m_lower=0.3, m_upper=1.2, m_solar=1,
                                    rectangular=0, approx=0, num_stars=45, num_phi=16, num_branches=2, random_seed=5),
    # disc with smooth mass, Kroupa with the full three-segment law
    "disc_kroupa_n70": dict(kappa_tot=0.2, kappa_star=0.15, shear=0.5, theta_star=1, mass_function="kroupa",
                            m_lower=0.01, m_upper=50, m_solar=1, rectangular=0, approx=1, num_stars=70,
                            num_phi=24, num_branches=3, random_seed=99),
}


def run_case(exe: str, name: str, params: dict, outdir: str) -> None:
    with tempfile.TemporaryDirectory() as tmp:
        prefix = tmp + "/"
        args = [exe] + sum([[OPTS[k], str(v)] for k, v in params.items()], []) + ["-wls", "1", "-o", prefix]
        subprocess.run(args, check=True)
        info = O.read_params(prefix + "ccf_ref_info.txt")
        sorted_sf = O.read_star_file(prefix + "ccf_stars.bin")
        gen_sf = O.read_star_file(prefix + "ccf_stars_unsorted.bin")
        np.savez_compressed(
            os.path.join(outdir, f"{name}.npz"),
            params=json.dumps(params),
            info=json.dumps(info),
            stars_generated=gen_sf["stars"],
            stars_sorted=sorted_sf["stars"],
            corner=np.array([sorted_sf["corner"].real, sorted_sf["corner"].imag]),
            ccs=O.read_array(prefix + "ccf_ccs.bin", is_complex=True),
            caustics=O.read_array(prefix + "ccf_caustics.bin", is_complex=True),
            errs=O.read_array(prefix + "ccf_errs.bin"),
            mu_length_scales=O.read_array(prefix + "ccf_mu_length_scales.bin"),
        )


def main() -> None:
    exe = O.build_reference()
    if exe is None:
        raise SystemExit("reference sources not present; fixtures can only be regenerated where they are")
    outdir = os.path.dirname(os.path.abspath(__file__))
    for name, params in CASES.items():
        run_case(exe, name, params, outdir)
        print("wrote", name)


if __name__ == "__main__":
    main()
