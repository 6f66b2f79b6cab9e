"""Amber prmtop input for the ATM path.

The reference's ABFE test builds its system from an Amber prmtop with OpenMM's
AmberPrmtopFile and createSystem (python/tests/test_abfe.py:36-60); the ATM force
re-evaluates that system's NonbondedForce.  This module reads what the
NonbondedForce needs from a prmtop — charges, Lennard-Jones sigma/epsilon per
atom from the type tables, the excluded 1-2 and 1-3 pairs and the scaled 1-4
pairs of the dihedral list (SCEE/SCNB, default 1.2 and 2.0), masses, residues,
default box — and builds a System laid out as the reference's test does
(NonbondedForce in group 1, ATMMetaForce over every particle in group 2,
re-evaluating group 1).  It also reads positions and box vectors from an OpenMM
State XML file (the test's equilibrated state).

Units: nm, e, kJ/mol (prmtop charges are e x 18.2223, lengths in Angstrom,
energies in kcal/mol).
"""
from __future__ import annotations

import re
from dataclasses import dataclass, field

import numpy as np

AMBER_CHARGE_SCALE = 18.2223
KCAL = 4.184


def read_prmtop_sections(path):
    """{FLAG: list of string tokens} for the fixed-width sections of a prmtop."""
    flags = {}
    name, width, items = None, None, None
    with open(path) as f:
        for line in f:
            if line.startswith("%FLAG"):
                if name is not None:
                    flags[name] = items
                name = line.split()[1]
                items = []
                width = None
            elif line.startswith("%FORMAT"):
                m = re.search(r"\((\d+)([aIE])(\d+)", line)
                width = int(m.group(3))
            elif line.startswith("%"):
                continue
            elif name is not None:
                s = line.rstrip("\n")
                for k in range(0, len(s), width):
                    tok = s[k:k + width].strip()
                    if tok:
                        items.append(tok)
        if name is not None:
            flags[name] = items
    return flags


@dataclass
class Prmtop:
    natom: int
    charge: np.ndarray       # e
    sigma: np.ndarray        # nm
    epsilon: np.ndarray      # kJ/mol
    mass: np.ndarray         # amu
    residue_start: np.ndarray  # first atom of each residue (plus natom at the end)
    residue_name: list
    exc_i: np.ndarray
    exc_j: np.ndarray
    exc_qq: np.ndarray       # e^2 (0 for exclusions)
    exc_sig: np.ndarray
    exc_eps: np.ndarray
    box: np.ndarray = field(default_factory=lambda: np.zeros(3))  # default box (nm), zeros if none

    def residue_atoms(self, k):
        """Atom indices of residue k (0-based)."""
        return np.arange(self.residue_start[k], self.residue_start[k + 1])


def read_prmtop(path):
    """Parse an Amber prmtop into the NonbondedForce description (see the module
    docstring): exceptions list the 1-2/1-3 exclusions first (chargeProd 0,
    epsilon 0), then the 1-4 pairs with chargeProd q_i q_j / SCEE, sigma the
    arithmetic mean and epsilon sqrt(e_i e_j) / SCNB, both in index order."""
    P = read_prmtop_sections(path)
    ptr = [int(x) for x in P["POINTERS"]]
    natom, ntypes = ptr[0], ptr[1]
    charge = np.array([float(x) for x in P["CHARGE"]]) / AMBER_CHARGE_SCALE
    atype = np.array([int(x) for x in P["ATOM_TYPE_INDEX"]]) - 1
    nbidx = np.array([int(x) for x in P["NONBONDED_PARM_INDEX"]])
    acoef = np.array([float(x) for x in P["LENNARD_JONES_ACOEF"]])
    bcoef = np.array([float(x) for x in P["LENNARD_JONES_BCOEF"]])
    # per-type sigma / epsilon from the diagonal of the A/B tables (A = 4 e s^12, B = 4 e s^6)
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
    mass = np.array([float(x) for x in P["MASS"]]) if "MASS" in P else np.zeros(natom)
    rstart = np.array([int(x) - 1 for x in P["RESIDUE_POINTER"]] + [natom])
    rname = list(P.get("RESIDUE_LABEL", []))

    def records(flag, width):
        v = [int(x) for x in P.get(flag, [])]
        return [v[k:k + width] for k in range(0, len(v), width)]

    excl = set()
    for rec in records("BONDS_INC_HYDROGEN", 3) + records("BONDS_WITHOUT_HYDROGEN", 3):
        i, j = abs(rec[0]) // 3, abs(rec[1]) // 3
        excl.add((min(i, j), max(i, j)))
    for rec in records("ANGLES_INC_HYDROGEN", 4) + records("ANGLES_WITHOUT_HYDROGEN", 4):
        i, j = abs(rec[0]) // 3, abs(rec[2]) // 3
        excl.add((min(i, j), max(i, j)))
        for a, b in ((rec[0], rec[1]), (rec[1], rec[2])):
            a, b = abs(a) // 3, abs(b) // 3
            excl.add((min(a, b), max(a, b)))
    scee = [float(x) for x in P.get("SCEE_SCALE_FACTOR", [])]
    scnb = [float(x) for x in P.get("SCNB_SCALE_FACTOR", [])]
    pairs14 = {}
    for rec in records("DIHEDRALS_INC_HYDROGEN", 5) + records("DIHEDRALS_WITHOUT_HYDROGEN", 5):
        if rec[2] < 0:  # negative third index: end-group interaction not computed for this term
            continue
        i, l = abs(rec[0]) // 3, abs(rec[3]) // 3
        key = (min(i, l), max(i, l))
        if key in excl:
            continue
        t = rec[4] - 1
        pairs14[key] = (scee[t] if scee else 1.2, scnb[t] if scnb else 2.0)
    ei, ej, eqq, esig, eeps = [], [], [], [], []
    for (i, j) in sorted(excl):
        ei.append(i)
        ej.append(j)
        eqq.append(0.0)
        esig.append(1.0)
        eeps.append(0.0)
    for (i, j), (ee, nb) in sorted(pairs14.items()):
        ei.append(i)
        ej.append(j)
        eqq.append(charge[i] * charge[j] / ee)
        esig.append(0.5 * (sigma[i] + sigma[j]))
        eeps.append(np.sqrt(epsilon[i] * epsilon[j]) / nb)
    box = np.zeros(3)
    if "BOX_DIMENSIONS" in P:
        box = np.array([float(x) for x in P["BOX_DIMENSIONS"]][1:4]) * 0.1
    return Prmtop(natom=natom, charge=charge, sigma=sigma, epsilon=epsilon, mass=mass, residue_start=rstart,
                  residue_name=rname, exc_i=np.array(ei, dtype=np.int32), exc_j=np.array(ej, dtype=np.int32),
                  exc_qq=np.array(eqq), exc_sig=np.array(esig), exc_eps=np.array(eeps), box=box)


def read_state_xml(path):
    """Positions (n x 3, nm) and orthorhombic box edges (nm) of an OpenMM State XML."""
    with open(path) as f:
        txt = f.read()
    box = []
    for tag in ("A", "B", "C"):
        m = re.search(r"<%s x=\"([^\"]+)\" y=\"([^\"]+)\" z=\"([^\"]+)\"" % tag, txt)
        box.append([float(m.group(1)), float(m.group(2)), float(m.group(3))])
    pos = [[float(m.group(1)), float(m.group(2)), float(m.group(3))]
           for m in re.finditer(r"<Position x=\"([^\"]+)\" y=\"([^\"]+)\" z=\"([^\"]+)\"", txt)]
    return np.array(pos), np.diag(np.array(box))


def system_from_prmtop(prm, ligand, displacement, params, cutoff=1.0, ewald_tol=5e-4, box=None,
                       nonbonded_group=1, atm_group=2):
    """System with the prmtop's NonbondedForce (PME) in ``nonbonded_group`` and an
    ATMMetaForce over every particle in ``atm_group``; the ``ligand`` atoms carry
    ``displacement`` (nm).  ``params``: lambda1, lambda2, alpha, u0, w0, umax,
    ubcore, acore, direction.  ``box``: default box edges (nm), else the prmtop's."""
    from .api import ATMMetaForce, NonbondedForce, System

    sys_ = System()
    for k in range(prm.natom):
        sys_.addParticle(float(prm.mass[k]) if prm.mass[k] > 0 else 1.0)
    L = np.asarray(prm.box if box is None else box, dtype=np.float64)
    sys_.setDefaultPeriodicBoxVectors((L[0], 0, 0), (0, L[1], 0), (0, 0, L[2]))
    nb = NonbondedForce()
    for k in range(prm.natom):
        nb.addParticle(prm.charge[k], prm.sigma[k], prm.epsilon[k])
    for k in range(len(prm.exc_i)):
        nb.addException(int(prm.exc_i[k]), int(prm.exc_j[k]), prm.exc_qq[k], prm.exc_sig[k], prm.exc_eps[k])
    nb.setNonbondedMethod(NonbondedForce.PME)
    nb.setCutoffDistance(cutoff)
    nb.setEwaldErrorTolerance(ewald_tol)
    nb.setForceGroup(nonbonded_group)
    sys_.addForce(nb)
    p = list(params)
    f = ATMMetaForce(*p, [nonbonded_group])
    d = np.asarray(displacement, dtype=np.float64)
    lig = set(int(i) for i in ligand)
    for k in range(prm.natom):
        if k in lig:
            f.addParticle(k, d[0], d[1], d[2])
        else:
            f.addParticle(k, 0.0, 0.0, 0.0)
    f.setForceGroup(atm_group)
    sys_.addForce(f)
    return sys_, nb, f
