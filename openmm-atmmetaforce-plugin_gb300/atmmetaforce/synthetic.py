"""Seeded synthetic ATM systems: water-like triples around one or two ligand chains.

These stand in for the workloads the ATM benchmark is quoted on (no public
dataset is involved).  Every array is produced from ``numpy.random.default_rng(seed)``
so the same seed gives the same system on any machine.

Geometry and parameters (all units nm, kJ/mol, e):
  - water O: q = -0.834, sigma 0.315, eps 0.636; H: q = +0.417, no LJ;
    O-H 0.09572 nm, H-O-H 104.52 deg, random orientation; O on a cubic lattice
    jittered by U[-0.02, 0.02] per coordinate; O-H and H-H pairs excluded;
  - ligand: a chain with 0.15 nm bonds, 111 deg bond angles and random
    dihedrals (a straight chain would not fit the smaller boxes), charges
    U[-0.5, 0.5] shifted to net zero, sigma U[0.25, 0.40], eps U[0.2, 0.9],
    1-2 and 1-3 pairs excluded;
  - lattice sites closer than 0.3 nm (minimum image) to a ligand atom, at its
    original or displaced position, are left empty, so that both ATM end states
    start from a solvent cavity (an equilibrated ATM set-up looks like this);
  - the ligand sits at the box origin; molecules are kept whole, not wrapped.
"""
from __future__ import annotations

import math
from dataclasses import dataclass, field

import numpy as np

NOCUTOFF, CUTOFF_NONPERIODIC, CUTOFF_PERIODIC, PME = 0, 1, 2, 4

WATER_O = (-0.834, 0.315, 0.636)
WATER_H = (0.417, 0.1, 0.0)
R_OH = 0.09572
HOH_DEG = 104.52


def pme_parameters(cutoff, tol, box, legal=False):
    """OpenMM's documented PME rule: alpha = sqrt(-ln(2 tol))/rc and
    n_d = ceil(2 alpha L_d / (3 tol^(1/5))) (at least 6); ``legal`` rounds up to a
    size with prime factors 2, 3, 5, 7 only."""
    alpha = math.sqrt(-math.log(2.0 * tol)) / cutoff
    grid = []
    for L in box:
        g = max(6, int(math.ceil(2.0 * alpha * L / (3.0 * tol ** 0.2))))
        if legal:
            while True:
                m = g
                for p in (2, 3, 5, 7):
                    while m % p == 0:
                        m //= p
                if m == 1:
                    break
                g += 1
        grid.append(g)
    return alpha, grid


@dataclass
class NonbondedSpec:
    """Plain-array description of a NonbondedForce (what the oracle and the
    context builder both consume)."""

    charge: np.ndarray
    sigma: np.ndarray
    epsilon: np.ndarray
    exc_i: np.ndarray
    exc_j: np.ndarray
    exc_qq: np.ndarray
    exc_sig: np.ndarray
    exc_eps: np.ndarray
    method: int
    cutoff: float
    box: np.ndarray
    eps_rf: float = 78.5
    # b_x, c_x, c_y of OpenMM's reduced triclinic box vectors a = (box0, 0, 0),
    # b = (b_x, box1, 0), c = (c_x, c_y, box2); zeros for an orthorhombic box
    tilt: tuple = (0.0, 0.0, 0.0)
    ewald_tol: float = 5e-4
    alpha: float = 0.0
    grid: tuple = (0, 0, 0)
    order: int = 5
    use_disp_corr: bool = False

    @property
    def n(self):
        return len(self.charge)


@dataclass
class ATMCase:
    spec: NonbondedSpec
    pos: np.ndarray        # (n, 3)
    displ: np.ndarray      # (n, 3)
    params: np.ndarray     # lambda1, lambda2, alpha, u0, w0, umax, ubcore, acore, direction
    ligands: list = field(default_factory=list)   # list of index arrays
    seed: int = 0
    name: str = ""

    @property
    def n(self):
        return len(self.pos)


PARAM_NAMES = ("ATMLambda1", "ATMLambda2", "ATMAlpha", "ATMU0", "ATMW0",
               "ATMUmax", "ATMUbcore", "ATMAcore", "ATMDirection")


def default_params(lambda1=0.5, lambda2=0.5, alpha=0.0, u0=0.0, w0=0.0,
                   umax=200.0, ubcore=100.0, acore=0.0625, direction=1.0):
    return np.array([lambda1, lambda2, alpha, u0, w0, umax, ubcore, acore, direction], dtype=np.float64)


def _rotation(rng):
    q = rng.normal(size=4)
    q /= np.linalg.norm(q)
    a, b, c, d = q
    return np.array([
        [a * a + b * b - c * c - d * d, 2 * (b * c - a * d), 2 * (b * d + a * c)],
        [2 * (b * c + a * d), a * a - b * b + c * c - d * d, 2 * (c * d - a * b)],
        [2 * (b * d - a * c), 2 * (c * d + a * b), a * a - b * b - c * c + d * d],
    ])


def _chain(rng, n, bond=0.15, angle_deg=111.0, min_sep=0.3):
    """Self-avoiding chain with fixed bonds and angles (NeRF placement): each
    dihedral is drawn at random until the new atom is at least ``min_sep`` from
    every atom three or more bonds away (or the best of 64 draws)."""
    th = math.radians(angle_deg)
    x = np.zeros((n, 3))
    if n > 1:
        x[1] = [bond, 0, 0]
    if n > 2:
        x[2] = x[1] + bond * np.array([-math.cos(th), math.sin(th), 0.0])
    for i in range(3, n):
        a, b, c = x[i - 3], x[i - 2], x[i - 1]
        bc = (c - b) / np.linalg.norm(c - b)
        nrm = np.cross(b - a, bc)
        nrm /= np.linalg.norm(nrm)
        m = np.stack([bc, np.cross(nrm, bc), nrm], axis=1)
        best, best_d = None, -1.0
        for _ in range(64):
            phi = rng.uniform(-math.pi, math.pi)
            d2 = np.array([-bond * math.cos(th), bond * math.sin(th) * math.cos(phi),
                           bond * math.sin(th) * math.sin(phi)])
            cand = c + m @ d2
            far = x[: i - 3]
            dmin = np.sqrt(((far - cand) ** 2).sum(axis=1)).min() if i > 3 else 1e9
            if dmin > best_d:
                best, best_d = cand, dmin
            if dmin >= min_sep:
                break
        x[i] = best
    return x - x.mean(axis=0)


def _ligand_params(rng, n):
    q = rng.uniform(-0.5, 0.5, n)
    q -= q.mean()
    sig = rng.uniform(0.25, 0.40, n)
    eps = rng.uniform(0.2, 0.9, n)
    return q, sig, eps


def _min_image(d, box):
    return d - box * np.round(d / box)


def box_vectors(box, tilt=(0.0, 0.0, 0.0)):
    """The 3 x 3 box vectors (rows a, b, c) of a box diagonal and its tilts."""
    return np.array([[box[0], 0.0, 0.0], [tilt[0], box[1], 0.0], [tilt[1], tilt[2], box[2]]], dtype=np.float64)


def min_image_triclinic(d, box, tilt):
    """OpenMM's minimum image in a reduced triclinic box: subtract c, then b,
    then a, each rounded to the nearest multiple (d: (..., 3))."""
    d = np.array(d, dtype=np.float64, copy=True)
    k = np.floor(d[..., 2] / box[2] + 0.5)
    d[..., 0] -= k * tilt[1]
    d[..., 1] -= k * tilt[2]
    d[..., 2] -= k * box[2]
    k = np.floor(d[..., 1] / box[1] + 0.5)
    d[..., 0] -= k * tilt[0]
    d[..., 1] -= k * box[1]
    k = np.floor(d[..., 0] / box[0] + 0.5)
    d[..., 0] -= k * box[0]
    return d


def water_ligand_box(n_total, box_edge, ligand_sizes, displacements, method, cutoff, seed,
                     params=None, eps_rf=78.5, ewald_tol=5e-4, ligand_centers=None, legal_grid=False,
                     use_disp_corr=False, name=""):
    """Build a cubic box of ``n_total`` atoms: the ligands plus (n_total - sum(L))/3 waters.

    ``displacements[k]`` is ligand k's displacement vector; ``ligand_centers[k]``
    its centroid (default: the origin for the first ligand, the first ligand's
    displaced site for the second one, as in a relative-binding swap).
    """
    rng = np.random.default_rng(seed)
    box = np.array([box_edge] * 3, dtype=np.float64)
    L_total = int(sum(ligand_sizes))
    n_water = int(round((n_total - L_total) / 3.0))
    if ligand_centers is None:
        ligand_centers = [np.zeros(3)]
        for k in range(1, len(ligand_sizes)):
            ligand_centers.append(np.asarray(ligand_centers[0]) + np.asarray(displacements[0]))

    lig_pos, lig_q, lig_s, lig_e = [], [], [], []
    for k, Lk in enumerate(ligand_sizes):
        x = _chain(rng, Lk) + np.asarray(ligand_centers[k], dtype=np.float64)
        q, s, e = _ligand_params(rng, Lk)
        lig_pos.append(x)
        lig_q.append(q)
        lig_s.append(s)
        lig_e.append(e)

    # lattice sites, cavities carved at both end states of every ligand
    avoid = np.concatenate([np.concatenate([x, x + np.asarray(d)]) for x, d in zip(lig_pos, displacements)])
    nside = int(math.ceil(n_water ** (1.0 / 3.0)))
    while True:
        g = (np.arange(nside) + 0.5) * (box_edge / nside)
        sites = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)
        keep = np.ones(len(sites), dtype=bool)
        for a in avoid:
            d = _min_image(sites - a, box)
            keep &= (d * d).sum(axis=1) >= 0.3 * 0.3
        if keep.sum() >= n_water:
            break
        nside += 1
    sites = sites[keep]
    chosen = np.sort(rng.choice(len(sites), size=n_water, replace=False))
    O = sites[chosen] + rng.uniform(-0.02, 0.02, size=(n_water, 3))
    half = math.radians(HOH_DEG) / 2.0
    h_local = np.array([[R_OH * math.sin(half), R_OH * math.cos(half), 0.0],
                        [-R_OH * math.sin(half), R_OH * math.cos(half), 0.0]])
    wat = np.zeros((n_water, 3, 3))
    for w in range(n_water):
        R = _rotation(rng)
        wat[w, 0] = O[w]
        wat[w, 1] = O[w] + R @ h_local[0]
        wat[w, 2] = O[w] + R @ h_local[1]

    n = 3 * n_water + L_total
    pos = np.zeros((n, 3))
    q = np.zeros(n)
    sig = np.zeros(n)
    eps = np.zeros(n)
    pos[: 3 * n_water] = wat.reshape(-1, 3)
    q[: 3 * n_water] = np.tile([WATER_O[0], WATER_H[0], WATER_H[0]], n_water)
    sig[: 3 * n_water] = np.tile([WATER_O[1], WATER_H[1], WATER_H[1]], n_water)
    eps[: 3 * n_water] = np.tile([WATER_O[2], WATER_H[2], WATER_H[2]], n_water)
    ei, ej = [], []
    base = np.arange(n_water) * 3
    for a, b in ((0, 1), (0, 2), (1, 2)):
        ei.append(base + a)
        ej.append(base + b)
    displ = np.zeros((n, 3))
    ligands = []
    off = 3 * n_water
    for k, Lk in enumerate(ligand_sizes):
        idx = np.arange(off, off + Lk)
        ligands.append(idx)
        pos[idx] = lig_pos[k]
        q[idx], sig[idx], eps[idx] = lig_q[k], lig_s[k], lig_e[k]
        displ[idx] = np.asarray(displacements[k], dtype=np.float64)
        for d in (1, 2):
            ei.append(idx[:-d])
            ej.append(idx[d:])
        off += Lk
    exc_i = np.concatenate(ei).astype(np.int32)
    exc_j = np.concatenate(ej).astype(np.int32)
    m = len(exc_i)
    alpha, grid = 0.0, (0, 0, 0)
    if method == PME:
        alpha, grid = pme_parameters(cutoff, ewald_tol, box, legal=legal_grid)
    spec = NonbondedSpec(charge=q, sigma=sig, epsilon=eps, exc_i=exc_i, exc_j=exc_j,
                         exc_qq=np.zeros(m), exc_sig=np.ones(m), exc_eps=np.zeros(m),
                         method=method, cutoff=cutoff, box=box, eps_rf=eps_rf, ewald_tol=ewald_tol,
                         alpha=alpha, grid=tuple(grid), use_disp_corr=use_disp_corr)
    if params is None:
        params = default_params()
    return ATMCase(spec=spec, pos=pos, displ=displ, params=np.asarray(params, dtype=np.float64),
                   ligands=ligands, seed=seed, name=name)


# ---------------------------------------------------------------------------
# The workloads the ATM benchmark and its parity cases are quoted on
# ---------------------------------------------------------------------------

# 22-state leg-1 softplus schedule: lambda1 ramps 0 -> 0.5 in 11 steps at
# lambda2 = 0.5, then lambda2 ramps 0.5 -> 1.0 in 11 steps at lambda1 = 0.5.
SCHEDULE_22 = np.array([(0.05 * r, 0.5) for r in range(11)] + [(0.5, 0.5 + 0.05 * r) for r in range(11)])


def abfe_rf_2394(seed=0):
    """2,394 atoms (790 waters + 24-atom ligand), 3.0 nm box, reaction field
    rc 0.9 nm eps_rf 78.5, displacement (1.5,1.5,1.5) nm, lambda 0.5, alpha 0."""
    return water_ligand_box(2394, 3.0, [24], [(1.5, 1.5, 1.5)], CUTOFF_PERIODIC, 0.9, seed,
                            params=default_params(0.5, 0.5, 0.0, 0.0, 0.0, 200.0, 100.0, 0.0625, 1.0),
                            name="abfe-rf-2394")


def abfe_pme_23558(seed=1, lambdas=(0.25, 0.25), alpha=0.0, u0=0.0):
    """23,558 atoms (7,838 waters + 44-atom ligand), 6.2 nm box, PME rc 0.9 nm,
    tolerance 5e-4 (grid 56^3), displacement (3.1,3.1,3.1) nm."""
    return water_ligand_box(23558, 6.2, [44], [(3.1, 3.1, 3.1)], PME, 0.9, seed,
                            params=default_params(lambdas[0], lambdas[1], alpha, u0, 0.0, 200.0, 100.0, 0.0625, 1.0),
                            name="abfe-pme-23558")


def abfe_pme_23558_x22(seed0=100):
    """22 independently seeded 23,558-atom PME replicas on the 22-state schedule
    (alpha 0.1 /(kJ/mol), u0 110 kJ/mol, w0 0)."""
    cases = []
    for r in range(22):
        l1, l2 = SCHEDULE_22[r]
        cases.append(abfe_pme_23558(seed=seed0 + r, lambdas=(l1, l2), alpha=0.1, u0=110.0))
    return cases


def abfe_pme_small(n_total, ligand, seed, box_edge=None, displ=2.0, cutoff=0.9):
    """A PME water box of about ``n_total`` atoms at the 23,558-atom density."""
    if box_edge is None:
        box_edge = (n_total / (23558 / 6.2 ** 3)) ** (1.0 / 3.0)
    return water_ligand_box(n_total, box_edge, [ligand], [(displ,) * 3], PME, cutoff, seed,
                            name=f"abfe-pme-{n_total}")


def mixed_batch_8(seed0=200):
    """8 boxes of 5,000 / 12,000 / 30,000 atoms (3/3/2) with 18/30/44-atom ligands."""
    sizes = [(5000, 18)] * 3 + [(12000, 30)] * 3 + [(30000, 44)] * 2
    out = []
    for k, (n, L) in enumerate(sizes):
        c = abfe_pme_small(n, L, seed0 + k)
        l1, l2 = SCHEDULE_22[(3 * k) % 22]
        c.params = default_params(l1, l2, 0.1, 110.0, 0.0, 200.0, 100.0, 0.0625, 1.0)
        out.append(c)
    return out


def adjoint_batch_8(seed0=300):
    """8 seeded 12,000-atom PME boxes with a 30-atom ligand displaced by
    (2,2,2) nm; lambdas U[0,0.5], alpha U[0,0.2], u0 U[50,150]."""
    rng = np.random.default_rng(seed0)
    out = []
    for k in range(8):
        c = abfe_pme_small(12000, 30, seed0 + 1 + k, displ=2.0)
        l1, l2 = rng.uniform(0, 0.5, 2)
        c.params = default_params(l1, l2, rng.uniform(0, 0.2), rng.uniform(50, 150), 0.0, 200.0, 100.0, 0.0625, 1.0)
        out.append(c)
    return out


def rbfe_pme_60000(seed=400):
    """60,000 atoms, 8.5 nm box, PME rc 1.0 nm; ligand A (30 atoms) displaced
    +(2.5,2.5,2.5) nm and ligand B (36 atoms), centred at A's displaced site,
    displaced -(2.5,2.5,2.5) nm."""
    return water_ligand_box(60000, 8.5, [30, 36], [(2.5, 2.5, 2.5), (-2.5, -2.5, -2.5)], PME, 1.0, seed,
                            params=default_params(0.25, 0.25, 0.1, 110.0, 0.0, 200.0, 100.0, 0.0625, 1.0),
                            name="rbfe-pme-60000")


# ---------------------------------------------------------------------------
# MD terms: the group-0 forces the reference's ABFE test integrates with the
# ATM force (python/tests/test_abfe.py:55-103)
# ---------------------------------------------------------------------------

MASS_O, MASS_H, MASS_LIG = 15.999, 1.008, 12.011
KCAL_A2 = 4.184 * 100.0  # kcal/mol/A^2 in kJ/mol/nm^2


@dataclass
class MDTerms:
    masses: np.ndarray                  # (n,)
    constraints: list                   # (i, j, distance)
    bonds: list                         # (i, j, length, k)
    angles: list                        # (i, j, l, angle, k)
    posres_particles: np.ndarray        # restrained "receptor" atoms
    posres_ref: np.ndarray              # (n, 3) reference positions
    posres_fc: float
    posres_tol: float
    posres_periodic: bool
    centroid: list                      # (g1, g2, kf, tol, offset)


def _angle(a, b, c):
    u, v = a - b, c - b
    return math.atan2(np.linalg.norm(np.cross(u, v)), float(np.dot(u, v)))


def md_terms(case, n_receptor=8, bond_k=2.5e5, angle_k=500.0, rigid_water=True):
    """Masses, rigid-water constraints, ligand bonds and angles at their built
    geometry, and the restraints of the reference's ABFE test: the ``n_receptor``
    water oxygens nearest the first ligand stand in for the receptor atoms (their
    molecules moved to the periodic image next to the ligand), held by flat-bottom
    position restraints (25 kcal/mol/A^2, 0.5 A) and joined to the ligand by a
    centroid restraint (25 kcal/mol/A^2, 5 A, offset = the starting centroid
    separation).  Returns (terms, positions)."""
    pos = case.pos.copy()
    n = case.n
    lig_all = np.concatenate(case.ligands) if case.ligands else np.zeros(0, dtype=int)
    n_water = (n - len(lig_all)) // 3
    box = case.spec.box
    masses = np.full(n, MASS_LIG)
    masses[: 3 * n_water] = np.tile([MASS_O, MASS_H, MASS_H], n_water)
    cons = []
    if rigid_water:
        d_hh = 2.0 * R_OH * math.sin(math.radians(HOH_DEG) / 2.0)
        for w in range(n_water):
            o = 3 * w
            cons += [(o, o + 1, R_OH), (o, o + 2, R_OH), (o + 1, o + 2, d_hh)]
    bonds, angles = [], []
    for lig in case.ligands:
        for a in range(len(lig) - 1):
            i, j = int(lig[a]), int(lig[a + 1])
            bonds.append((i, j, float(np.linalg.norm(pos[j] - pos[i])), bond_k))
        for a in range(len(lig) - 2):
            i, j, l = int(lig[a]), int(lig[a + 1]), int(lig[a + 2])
            angles.append((i, j, l, _angle(pos[i], pos[j], pos[l]), angle_k))
    rec = np.zeros(0, dtype=int)
    centroid = []
    if case.ligands and n_water >= n_receptor > 0:
        lig = case.ligands[0]
        c_lig = (masses[lig, None] * pos[lig]).sum(0) / masses[lig].sum()
        O = 3 * np.arange(n_water)
        d = _min_image(pos[O] - c_lig, box)
        near = np.argsort((d * d).sum(1), kind="stable")[:n_receptor]
        for w in near:
            o = int(O[w])
            shift = d[w] - (pos[o] - c_lig)  # image of the oxygen next to the ligand
            pos[o:o + 3] += shift
        rec = np.sort(O[near])
        c_rec = (masses[rec, None] * pos[rec]).sum(0) / masses[rec].sum()
        centroid.append((np.asarray(lig, dtype=int), rec, 25.0 * KCAL_A2, 0.5, c_lig - c_rec))
    terms = MDTerms(masses=masses, constraints=cons, bonds=bonds, angles=angles, posres_particles=rec,
                    posres_ref=pos.copy(), posres_fc=25.0 * KCAL_A2, posres_tol=0.05, posres_periodic=True,
                    centroid=centroid)
    return terms, pos


def md_terms_ligand_centroid(case, kf=25.0, tol=0.15, bond_k=2.5e5, angle_k=500.0, rigid_water=True):
    """MD terms of the benchmark's plain-ATM MD runs: masses, rigid waters, each
    ligand's bonds and angles at their built geometry, and a flat-bottom harmonic
    restraint of every ligand atom to its ligand's mass-weighted centroid,
    (kf/2) step(d - tol)(d - tol)^2 with d = |x_i - c_ligand| (kf in kJ/mol/nm^2,
    tol in nm; each one a centroid restraint of the atom against its ligand, no
    periodic image).  No receptor, so no position restraints.  Returns (terms,
    positions)."""
    terms, pos = md_terms(case, n_receptor=0, bond_k=bond_k, angle_k=angle_k, rigid_water=rigid_water)
    cent = []
    for lig in case.ligands:
        g2 = np.asarray(lig, dtype=int)
        for i in g2:
            cent.append((np.array([int(i)]), g2, float(kf), float(tol), np.zeros(3)))
    terms.centroid = cent
    return terms, pos



def triclinic_water_ligand_box(n_total, box, tilt, ligand_sizes, displacements, method, cutoff, seed, params=None,
                               eps_rf=78.5, ewald_tol=5e-4, name=""):
    """A triclinic box (OpenMM's reduced form: box diagonal ``box``, tilts b_x,
    c_x, c_y) of ``n_total`` atoms with the distributions of
    ``water_ligand_box``: water oxygens on a jittered lattice of fractional
    coordinates mapped through the box vectors (rigid water geometry kept),
    cavities of 0.3 nm (triclinic minimum image) around every ligand atom at both
    end states.  The PME grid follows OpenMM's rule on the box diagonal."""
    rng = np.random.default_rng(seed)
    box = np.asarray(box, dtype=np.float64)
    tilt = np.asarray(tilt, dtype=np.float64)
    B = box_vectors(box, tilt)
    L_total = int(sum(ligand_sizes))
    n_water = int(round((n_total - L_total) / 3.0))
    centers = [np.zeros(3)]
    for k in range(1, len(ligand_sizes)):
        centers.append(centers[0] + np.asarray(displacements[0]))
    lig_pos, lig_q, lig_s, lig_e = [], [], [], []
    for k, Lk in enumerate(ligand_sizes):
        lig_pos.append(_chain(rng, Lk) + centers[k])
        q, sg, ep = _ligand_params(rng, Lk)
        lig_q.append(q)
        lig_s.append(sg)
        lig_e.append(ep)
    avoid = np.concatenate([np.concatenate([x, x + np.asarray(d)]) for x, d in zip(lig_pos, displacements)])
    nside = int(math.ceil(n_water ** (1.0 / 3.0)))
    while True:
        g = (np.arange(nside) + 0.5) / nside
        frac = np.stack(np.meshgrid(g, g, g, indexing="ij"), axis=-1).reshape(-1, 3)
        sites = frac @ B
        keep = np.ones(len(sites), dtype=bool)
        for a_ in avoid:
            d = min_image_triclinic(sites - a_, box, tilt)
            keep &= (d * d).sum(axis=1) >= 0.3 * 0.3
        if keep.sum() >= n_water:
            break
        nside += 1
    sites = sites[keep]
    chosen = np.sort(rng.choice(len(sites), size=n_water, replace=False))
    O = sites[chosen] + rng.uniform(-0.02, 0.02, size=(n_water, 3))
    half = math.radians(HOH_DEG) / 2.0
    h_local = np.array([[R_OH * math.sin(half), R_OH * math.cos(half), 0.0],
                        [-R_OH * math.sin(half), R_OH * math.cos(half), 0.0]])
    n = 3 * n_water + L_total
    pos = np.zeros((n, 3))
    for w in range(n_water):
        R = _rotation(rng)
        pos[3 * w] = O[w]
        pos[3 * w + 1] = O[w] + R @ h_local[0]
        pos[3 * w + 2] = O[w] + R @ h_local[1]
    q = np.zeros(n)
    sig = np.zeros(n)
    eps = np.zeros(n)
    q[: 3 * n_water] = np.tile([WATER_O[0], WATER_H[0], WATER_H[0]], n_water)
    sig[: 3 * n_water] = np.tile([WATER_O[1], WATER_H[1], WATER_H[1]], n_water)
    eps[: 3 * n_water] = np.tile([WATER_O[2], WATER_H[2], WATER_H[2]], n_water)
    ei, ej = [], []
    base = np.arange(n_water) * 3
    for a_, b_ in ((0, 1), (0, 2), (1, 2)):
        ei.append(base + a_)
        ej.append(base + b_)
    displ = np.zeros((n, 3))
    ligands = []
    off = 3 * n_water
    for k, Lk in enumerate(ligand_sizes):
        idx = np.arange(off, off + Lk)
        ligands.append(idx)
        pos[idx] = lig_pos[k]
        q[idx], sig[idx], eps[idx] = lig_q[k], lig_s[k], lig_e[k]
        displ[idx] = np.asarray(displacements[k], dtype=np.float64)
        for d in (1, 2):
            ei.append(idx[:-d])
            ej.append(idx[d:])
        off += Lk
    exc_i = np.concatenate(ei).astype(np.int32)
    exc_j = np.concatenate(ej).astype(np.int32)
    m = len(exc_i)
    alpha, grid = 0.0, (0, 0, 0)
    if method == PME:
        alpha, grid = pme_parameters(cutoff, ewald_tol, box)
    spec = NonbondedSpec(charge=q, sigma=sig, epsilon=eps, exc_i=exc_i, exc_j=exc_j, exc_qq=np.zeros(m),
                         exc_sig=np.ones(m), exc_eps=np.zeros(m), method=method, cutoff=cutoff, box=box,
                         eps_rf=eps_rf, ewald_tol=ewald_tol, alpha=alpha, grid=tuple(grid),
                         tilt=tuple(float(t) for t in tilt))
    if params is None:
        params = default_params()
    return ATMCase(spec=spec, pos=pos, displ=displ, params=np.asarray(params, dtype=np.float64), ligands=ligands,
                   seed=seed, name=name)
