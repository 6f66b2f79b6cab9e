"""Pin of the oracle against the reference's own ATM test.

python/tests/test_abfe.py:147-150 asserts that on TEMOA-G1 (guest displaced by
22 A, lambda 0.5) the perturbation energy is 58.2 kJ/mol within 0.1.  The
fixture tests/golden/temoa_g1.npz is extracted from that test's inputs by
tests/golden/make_temoa_fixture.py.
"""
import os

import numpy as np
import pytest

import oracle as O
from atmmetaforce import synthetic as S

FIX = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden", "temoa_g1.npz")


def temoa_spec(legal):
    z = np.load(FIX)
    alpha, grid = S.pme_parameters(float(z["cutoff"]), float(z["ewald_tol"]), z["box_default"], legal=legal)
    spec = S.NonbondedSpec(charge=z["charge"], sigma=z["sigma"], epsilon=z["epsilon"], exc_i=z["exc_i"],
                           exc_j=z["exc_j"], exc_qq=z["exc_qq"], exc_sig=z["exc_sig"], exc_eps=z["exc_eps"],
                           method=S.PME, cutoff=float(z["cutoff"]), box=z["box"], alpha=alpha, grid=tuple(grid),
                           use_disp_corr=True)
    d = np.zeros_like(z["pos"])
    d[z["ligand"]] = z["displacement"]
    return z, spec, d


@pytest.mark.parametrize("legal", [False, True], ids=["reference-grid", "fft-legal-grid"])
def test_temoa_perturbation_energy_matches_reference_test(legal):
    z, spec, d = temoa_spec(legal)
    O.set_threads(4)
    try:
        r = O.atm_eval(spec, z["pos"], d, z["params"])
    finally:
        O.set_threads(1)
    assert abs(r["usc"] - float(z["expected_u"])) <= float(z["expected_u_atol"]), r["usc"]
    # below ubcore the soft-core map is the identity
    assert r["usc"] == r["u"]
