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

Run from the repository root:  python tests/golden/make_temoa_fixture.py
(reads the reference checkout; the fixture it writes is committed, so tests do
not need the reference at run time).
"""
from __future__ import annotations

import os
import re
import sys

import numpy as np

REF = os.environ.get("ATM_REFERENCE_DIR", "/root/reference")
SRC = os.path.join(REF, "python", "tests")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "temoa_g1.npz")

AMBER_CHARGE_SCALE = 18.2223  # prmtop charges are e * 18.2223
KCAL = 4.184


def read_prmtop(path):
    """Return {FLAG: list of tokens} for the fixed-format sections of a prmtop."""
    flags = {}
    name, fmt_width, items = None, None, None
    with open(path) as f:
        for line in f:
            if line.startswith("%FLAG"):
                if name is not None:
                    flags[name] = items
                name = line.split()[1]
                items = []
                fmt_width = None
            elif line.startswith("%FORMAT"):
                m = re.search(r"\((\d+)([aIE])(\d+)", line)
                fmt_width = int(m.group(3))
            elif line.startswith("%"):
                continue
            elif name is not None:
                s = line.rstrip("\n")
                for k in range(0, len(s), fmt_width):
                    tok = s[k:k + fmt_width].strip()
                    if tok:
                        items.append(tok)
        if name is not None:
            flags[name] = items
    return flags


def read_state_xml(path):
    pos, box = [], []
    with open(path) as f:
        txt = f.read()
    for tag in ("A", "B", "C"):
        m = re.search(r"<%s x=\"([^\"]+)\" y=\"([^\"]+)\" z=\"([^\"]+)\"" % tag, txt)
        box.append([float(m.group(1)), float(m.group(2)), float(m.group(3))])
    for m in re.finditer(r"<Position x=\"([^\"]+)\" y=\"([^\"]+)\" z=\"([^\"]+)\"", txt):
        pos.append([float(m.group(1)), float(m.group(2)), float(m.group(3))])
    return np.array(pos), np.array(box)


def main():
    P = read_prmtop(os.path.join(SRC, "temoa-g1.prmtop"))
    ptr = [int(x) for x in P["POINTERS"]]
    natom, ntypes = ptr[0], ptr[1]
    charge = np.array([float(x) for x in P["CHARGE"]]) / AMBER_CHARGE_SCALE
    atype = np.array([int(x) for x in P["ATOM_TYPE_INDEX"]]) - 1
    nbidx = np.array([int(x) for x in P["NONBONDED_PARM_INDEX"]])
    acoef = np.array([float(x) for x in P["LENNARD_JONES_ACOEF"]])
    bcoef = np.array([float(x) for x in P["LENNARD_JONES_BCOEF"]])
    # per-type sigma/epsilon from the diagonal of the A/B tables (A = 4 e s^12, B = 4 e s^6)
    tsig = np.ones(ntypes)
    teps = np.zeros(ntypes)
    for t in range(ntypes):
        k = nbidx[ntypes * t + t] - 1
        A, B = acoef[k], bcoef[k]
        if A > 0 and B > 0:
            tsig[t] = (A / B) ** (1.0 / 6.0) * 0.1
            teps[t] = B * B / (4.0 * A) * KCAL
    sigma = tsig[atype]
    epsilon = teps[atype]

    # residues: the guest is residue 2 (1-based), as test_abfe.py:26,47-50 selects it
    rptr = [int(x) - 1 for x in P["RESIDUE_POINTER"]] + [natom]
    ligand = np.arange(rptr[1], rptr[2])

    # exclusions and 1-4 pairs from bonds, angles, dihedrals
    def triples(flag, width):
        v = [int(x) for x in P[flag]]
        return [v[k:k + width] for k in range(0, len(v), width)]

    excl = set()
    for rec in triples("BONDS_INC_HYDROGEN", 3) + triples("BONDS_WITHOUT_HYDROGEN", 3):
        i, j = abs(rec[0]) // 3, abs(rec[1]) // 3
        excl.add((min(i, j), max(i, j)))
    for rec in triples("ANGLES_INC_HYDROGEN", 4) + triples("ANGLES_WITHOUT_HYDROGEN", 4):
        i, j = abs(rec[0]) // 3, abs(rec[2]) // 3
        excl.add((min(i, j), max(i, j)))
        for a, b in ((rec[0], rec[1]), (rec[1], rec[2])):
            a, b = abs(a) // 3, abs(b) // 3
            excl.add((min(a, b), max(a, b)))
    scee = [float(x) for x in P.get("SCEE_SCALE_FACTOR", [])]
    scnb = [float(x) for x in P.get("SCNB_SCALE_FACTOR", [])]
    pairs14 = {}
    for rec in triples("DIHEDRALS_INC_HYDROGEN", 5) + triples("DIHEDRALS_WITHOUT_HYDROGEN", 5):
        if rec[2] < 0:  # end-group interactions not computed for this term
            continue
        i, l = abs(rec[0]) // 3, abs(rec[3]) // 3
        key = (min(i, l), max(i, l))
        if key in excl:
            continue
        t = rec[4] - 1
        pairs14[key] = (scee[t] if scee else 1.2, scnb[t] if scnb else 2.0)
    ei, ej, eqq, esig, eeps = [], [], [], [], []
    for (i, j) in sorted(excl):
        ei.append(i); ej.append(j); eqq.append(0.0); esig.append(1.0); eeps.append(0.0)
    for (i, j), (ee, nb) in sorted(pairs14.items()):
        ei.append(i); ej.append(j)
        eqq.append(charge[i] * charge[j] / ee)
        esig.append(0.5 * (sigma[i] + sigma[j]))
        eeps.append(np.sqrt(epsilon[i] * epsilon[j]) / nb)

    box_default = np.array([float(x) for x in P["BOX_DIMENSIONS"]][1:4]) * 0.1
    pos, box = read_state_xml(os.path.join(SRC, "temoa-g1-equil.xml"))
    assert pos.shape == (natom, 3), pos.shape
    np.savez_compressed(
        OUT,
        pos=pos, box=np.diag(box), box_default=box_default,
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
    print("wrote", OUT, "atoms", natom, "guest", len(ligand), "exceptions", len(ei),
          "box", np.diag(box).tolist(), "default box", box_default.tolist())


if __name__ == "__main__":
    sys.exit(main())
