"""Generate tests/golden/temoa_g1.npz from the reference's ABFE test inputs.

The reference's only numeric pin for the ATM path is python/tests/test_abfe.py:147-150:
on TEMOA-G1 (8,479 atoms, guest = residue 2, displaced by 22 A along each
axis, lambda 0.5, alpha 0) the perturbation energy is 58.2 +- 0.1 kJ/mol.  That
value depends only on the NonbondedForce (PME, 1 nm cutoff, Amber parameters)
in force group 1.  This script extracts what that force needs from the test's
Amber prmtop and equilibrated OpenMM state XML:

  positions (nm) and box (nm) of the state XML, the default box of the prmtop
  (which fixes the PME grid at context creation), per-atom charge (e), sigma
  (nm), epsilon (kJ/mol), the guest's atom indices, and the exception list
  (1-2/1-3 exclusions, scaled 1-4 pairs).

Run from the repository root with the reference checkout named explicitly:
  ATM_REFERENCE_DIR=<reference checkout> python tests/golden/make_temoa_fixture.py
or  python tests/golden/make_temoa_fixture.py <reference checkout> [out.npz]
(the fixture it writes is committed, so tests do not need the reference at run
time).
"""
from __future__ import annotations

import os
import sys

import numpy as np

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "temoa_g1.npz")

KCAL = 4.184

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, os.path.join(ROOT, "openmm-atmmetaforce-plugin_gb300"))
from atmmetaforce.amber import read_prmtop, read_state_xml  # noqa: E402


def main(ref, out=OUT):
    src = os.path.join(ref, "python", "tests")
    prm = read_prmtop(os.path.join(src, "temoa-g1.prmtop"))
    natom = prm.natom
    # residues: the guest is residue 2 (1-based), as test_abfe.py:26,47-50 selects it
    ligand = prm.residue_atoms(1)
    pos, box = read_state_xml(os.path.join(src, "temoa-g1-equil.xml"))
    assert pos.shape == (natom, 3), pos.shape
    charge, sigma, epsilon, box_default = prm.charge, prm.sigma, prm.epsilon, prm.box
    ei, ej, eqq, esig, eeps = prm.exc_i, prm.exc_j, prm.exc_qq, prm.exc_sig, prm.exc_eps
    np.savez_compressed(
        out,
        pos=pos, box=box, box_default=box_default,
        charge=charge, sigma=sigma, epsilon=epsilon, ligand=ligand.astype(np.int32),
        exc_i=np.array(ei, dtype=np.int32), exc_j=np.array(ej, dtype=np.int32),
        exc_qq=np.array(eqq), exc_sig=np.array(esig), exc_eps=np.array(eeps),
        # test_abfe.py:22-35: lambda 0.5, alpha 0, u0 0, w0 0, umax 200 kcal/mol,
        # ubcore 100 kcal/mol, acore 1/16, direction 1, displacement 22 A
        params=np.array([0.5, 0.5, 0.0, 0.0, 0.0, 200.0 * KCAL, 100.0 * KCAL, 0.0625, 1.0]),
        displacement=np.array([2.2, 2.2, 2.2]),
        cutoff=np.array(1.0), ewald_tol=np.array(5e-4),
        expected_u=np.array(58.2), expected_u_atol=np.array(0.1),
    )
    print("wrote", out, "atoms", natom, "guest", len(ligand), "exceptions", len(ei),
          "box", box.tolist(), "default box", box_default.tolist())


if __name__ == "__main__":
    ref = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("ATM_REFERENCE_DIR")
    if not ref:
        sys.exit("name the reference checkout: ATM_REFERENCE_DIR=<dir> or the first argument")
    sys.exit(main(ref, sys.argv[2] if len(sys.argv) > 2 else OUT))
