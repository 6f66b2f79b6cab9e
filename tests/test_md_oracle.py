"""CPU checks of the MD oracle: Philox known answers, group-0 forces against
finite differences, SHAKE, and energy conservation of the leapfrog step."""
import math

import numpy as np
import pytest

import md_oracle as M
from atmmetaforce import synthetic as S


def test_philox_known_answers():
    # Known-answer vectors of Philox4x32-10 published with the Random123 library.
    cases = [
        ((0, 0, 0, 0), (0, 0), (0x6627E8D5, 0xE169C58D, 0xBC57AC4C, 0x9B00DBD8)),
        ((0xFFFFFFFF,) * 4, (0xFFFFFFFF,) * 2, (0x408F276D, 0x41C83B0E, 0xA20BC7C6, 0x6D5451FD)),
        ((0x243F6A88, 0x85A308D3, 0x13198A2E, 0x03707344), (0xA4093822, 0x299F31D0),
         (0xD16CFE09, 0x94FDCCEB, 0x5001E420, 0x24126EA1)),
    ]
    for ctr, key, want in cases:
        got = M.philox4x32_10(np.array([ctr], dtype=np.uint64), np.array([key], dtype=np.uint64))[0]
        assert tuple(int(x) for x in got) == want


def test_normals_are_standard():
    z = M.normals3(200000, 7, M.RNG_THERMOSTAT, 12345)
    assert abs(z.mean()) < 0.01
    assert abs(z.var() - 1.0) < 0.01
    assert abs(np.corrcoef(z[:, 0], z[:, 1])[0, 1]) < 0.01
    # different steps, streams and seeds give different draws
    assert not np.array_equal(z, M.normals3(200000, 8, M.RNG_THERMOSTAT, 12345))
    assert not np.array_equal(z, M.normals3(200000, 7, M.RNG_VELOCITIES, 12345))
    assert not np.array_equal(z, M.normals3(200000, 7, M.RNG_THERMOSTAT, 12346))


@pytest.fixture(scope="module")
def small():
    case = S.abfe_pme_small(1200, 12, seed=7)
    terms, pos = S.md_terms(case)
    return case, terms, pos


def test_md_terms_layout(small):
    case, terms, pos = small
    nw = (case.n - 12) // 3
    assert len(terms.constraints) == 3 * nw
    assert len(terms.bonds) == 11 and len(terms.angles) == 10
    assert len(terms.posres_particles) == 8 and len(terms.centroid) == 1
    # the receptor molecules were moved next to the ligand, whole
    g1, g2, kf, tol, off = terms.centroid[0]
    c1 = pos[g1].mean(0)
    assert np.all(np.linalg.norm(pos[g2] - c1, axis=1) < 1.0)
    for i, j, d in terms.constraints:
        assert abs(np.linalg.norm(pos[i] - pos[j]) - d) < 1e-9
    E, F = M.group0(pos, terms, case.spec.box)
    assert abs(E) < 1e-9  # everything starts at its minimum


def test_group0_forces_match_finite_differences(small):
    case, terms, pos = small
    rng = np.random.default_rng(3)
    x = pos.copy()
    lig = case.ligands[0]
    x[lig] += rng.normal(scale=0.02, size=(len(lig), 3))
    x[terms.posres_particles] += rng.normal(scale=0.1, size=(len(terms.posres_particles), 3))
    x[lig] += 0.7  # centroid restraint beyond its 0.5 nm tolerance
    E, F = M.group0(x, terms, case.spec.box)
    assert E > 1.0
    atoms = list(lig) + list(terms.posres_particles)
    h = 1e-6
    for a in atoms:
        for k in range(3):
            xp, xm = x.copy(), x.copy()
            xp[a, k] += h
            xm[a, k] -= h
            fd = -(M.group0(xp, terms, case.spec.box)[0] - M.group0(xm, terms, case.spec.box)[0]) / (2 * h)
            assert abs(fd - F[a, k]) <= 1e-5 * max(1.0, abs(fd)), (a, k, fd, F[a, k])


def test_shake_restores_constraints(small):
    case, terms, pos = small
    rng = np.random.default_rng(5)
    inv_m = 1.0 / terms.masses
    clusters = M.constraint_clusters(terms.constraints, case.n)
    assert len(clusters) == len(terms.constraints) // 3
    xn = pos + rng.normal(scale=0.003, size=pos.shape)
    xs = M.shake(pos, xn, inv_m, clusters)
    for i, j, d in terms.constraints:
        r = np.linalg.norm(xs[i] - xs[j])
        assert abs(r * r - d * d) <= 2.5e-10 * d * d
    # the correction of each cluster moves its centre of mass not at all
    for atoms, _ in clusters[:50]:
        m = terms.masses[atoms]
        assert np.allclose((m[:, None] * xs[atoms]).sum(0), (m[:, None] * xn[atoms]).sum(0), atol=1e-12)


def test_verlet_conserves_energy_on_bonded_chains():
    # two ligand chains and nothing else: leapfrog Verlet (gamma = 0) keeps
    # bonds + angles + kinetic energy constant to O(dt^2)
    rng = np.random.default_rng(9)
    chain = S._chain(rng, 10)
    pos = np.concatenate([chain, chain + 1.0])
    ligs = [np.arange(10), np.arange(10, 20)]
    case = S.ATMCase(spec=None, pos=pos, displ=np.zeros_like(pos), params=S.default_params(), ligands=ligs)

    class _Spec:
        box = np.array([5.0, 5.0, 5.0])

    case.spec = _Spec()
    terms, x = S.md_terms(case, n_receptor=0, rigid_water=False)
    x = x + rng.normal(scale=0.005, size=x.shape)
    inv_m = 1.0 / terms.masses
    v = M.velocities_at(300.0, inv_m, 4)
    dt = 0.0005
    energies = []
    for step in range(400):
        E, F = M.group0(x, terms, case.spec.box)
        energies.append(E + M.kinetic(v, F, inv_m, dt))
        x, v = M.langevin_step(x, v, F, inv_m, 0.0, 0.0, dt, 1, step, [])
    energies = np.array(energies)
    assert energies.std() < 2e-3 * abs(energies.mean()) + 0.05, (energies.std(), energies.mean())
    assert abs(energies[-50:].mean() - energies[:50].mean()) < 0.05


def test_langevin_noise_and_friction_limits(small):
    case, terms, pos = small
    inv_m = 1.0 / terms.masses
    clusters = M.constraint_clusters(terms.constraints, case.n)
    v0 = M.velocities_at(300.0, inv_m, 2)
    f = np.zeros_like(pos)
    # gamma = 0 and zero force: free flight, velocities unchanged except along constraints
    x1, v1 = M.langevin_step(pos, v0, f, inv_m, 300.0, 0.0, 1e-4, 0, 0, [])
    assert np.allclose(v1, v0, rtol=0, atol=1e-9)  # (x + dt v - x)/dt rounds at ~1e-12
    # huge friction: velocities follow the noise alone, Maxwell-Boltzmann at T
    x2, v2 = M.langevin_step(pos, v0, f, inv_m, 300.0, 1e6, 0.002, 0, 0, [])
    ke = 0.5 * ((v2 * v2).sum(1) / inv_m).sum()
    assert abs(ke / (1.5 * case.n * M.KB * 300.0) - 1.0) < 0.05
    # constrained step keeps the constraints
    x3, v3 = M.langevin_step(pos, v0, f, inv_m, 300.0, 1.0, 0.002, 0, 0, clusters)
    for i, j, d in terms.constraints[:300]:
        assert abs(np.linalg.norm(x3[i] - x3[j]) - d) < 1e-9


def test_velocity_projection_removes_constraint_components(small):
    case, terms, pos = small
    inv_m = 1.0 / terms.masses
    clusters = M.constraint_clusters(terms.constraints, case.n)
    v = M.velocities_at(300.0, inv_m, 8)
    w = M.project_velocities(pos, v, inv_m, clusters)
    for i, j, d in terms.constraints:
        r = pos[i] - pos[j]
        assert abs(float((w[i] - w[j]) @ r)) <= 1e-10 * d * (np.linalg.norm(w[i]) + np.linalg.norm(w[j]))
    # momentum of each cluster is kept; kinetic energy only goes down
    for atoms, _ in clusters[:50]:
        m = terms.masses[atoms]
        assert np.allclose((m[:, None] * w[atoms]).sum(0), (m[:, None] * v[atoms]).sum(0), atol=1e-12)
    ke = lambda u: 0.5 * (terms.masses[:, None] * u * u).sum()
    assert ke(w) < ke(v)
    # the projected draw has the temperature of the unconstrained degrees of freedom
    dof = 3 * case.n - len(terms.constraints)
    assert abs(2 * ke(w) / (dof * M.KB) / 300.0 - 1.0) < 0.08
