"""Langevin MD driver on the GPU against the FP64 MD oracle.

Tolerances: the integrator, SHAKE and the Philox noise are FP64 on both sides,
so one step from the same forces agrees to rounding (positions 1e-10 nm,
velocities 1e-7 nm/ps; the FP32 Box-Muller noise differs by 1-2 ulp between
CUDA's logf/sincospif and numpy); rigid waters are solved by SETTLE on the GPU and
by converged SHAKE in the oracle; forces and energies carry the FP32 pair arithmetic of
the ATM evaluation (force RMS relative 1e-4, energy 2e-6 of the term sum).
"""
import os

import numpy as np
import pytest

import atmmetaforce as atm
import md_oracle as M
import oracle as O
from atmmetaforce import synthetic as S

pytestmark = pytest.mark.gpu


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


if not _has_gpu():
    pytest.skip("no CUDA device", allow_module_level=True)


@pytest.fixture(scope="module", autouse=True)
def _threads():
    O.set_threads(min(16, os.cpu_count() or 1))
    yield
    O.set_threads(1)


def _case(seed=7, n=1200, lig=12):
    case = S.abfe_pme_small(n, lig, seed=seed)
    case.params = S.default_params(0.3, 0.6, 0.1, 20.0, 0.0, 200.0, 100.0, 0.0625, 1.0)
    terms, pos = S.md_terms(case)
    case.pos = pos
    return case, terms


def _sim(case, terms, T=300.0, gamma=1.0, dt=0.002, seed=5, props=None):
    sys_, _, _ = atm.md_system_from_case(case, terms)
    integ = atm.LangevinIntegrator(T, gamma, dt)
    integ.setRandomNumberSeed(seed)
    sim = atm.Simulation(sys_, integ, 0, props)
    sim.setPositions(case.pos)
    return sim, integ


def _oracle_forces(case, terms, x):
    ref = O.atm_eval(case.spec, x, case.displ, case.params)
    E0, F0 = M.group0(x, terms, case.spec.box)
    return ref["energy"] + E0, ref["forces"] + F0


def test_velocities_and_one_step_match_oracle():
    case, terms = _case()
    sim, integ = _sim(case, terms)
    sim.setVelocitiesToTemperature(300.0, 11)
    s0 = sim.getState(getPositions=True, getVelocities=True, getForces=True, getEnergy=True)
    inv_m = 1.0 / terms.masses
    clusters = M.constraint_clusters(terms.constraints, case.n)
    v0 = M.velocities_at(300.0, inv_m, 11, x=case.pos, clusters=clusters)
    np.testing.assert_allclose(s0.getVelocities(), v0, rtol=0, atol=1e-6)
    # forces and energy at the start against the FP64 oracle
    E_ref, F_ref = _oracle_forces(case, terms, case.pos)
    F = s0.getForces()
    assert np.sqrt(((F - F_ref) ** 2).sum() / (F_ref ** 2).sum()) <= 1e-4
    _, _, T = O.nonbonded(case.spec, case.pos, forces=False)
    assert abs(s0.getPotentialEnergy() - E_ref) <= 2e-6 * (sum(abs(v) for v in T.values()) + 1.0)
    ke = M.kinetic(s0.getVelocities(), F, inv_m, 0.002, case.pos, clusters)
    assert abs(s0.getKineticEnergy() - ke) <= 1e-9 * ke
    # one step: the oracle step from the GPU's own forces
    sim.step(1)
    s1 = sim.getState(getPositions=True, getVelocities=True)
    # from the GPU's velocities (its FP32 Box-Muller draws differ from numpy's by an ulp)
    x1, v1 = M.langevin_step(case.pos, s0.getVelocities(), F, inv_m, 300.0, 1.0, 0.002, 5, 0, clusters)
    np.testing.assert_allclose(s1.getPositions(), x1, rtol=0, atol=1e-10)
    np.testing.assert_allclose(s1.getVelocities(), v1, rtol=0, atol=1e-7)
    assert sim.info()["steps"] == 1


def test_five_steps_track_oracle_trajectory():
    case, terms = _case(seed=8)
    sim, _ = _sim(case, terms, gamma=2.0, dt=0.001, seed=9)
    sim.setVelocitiesToTemperature(300.0, 3)
    inv_m = 1.0 / terms.masses
    clusters = M.constraint_clusters(terms.constraints, case.n)
    x, v = case.pos.copy(), M.velocities_at(300.0, inv_m, 3, x=case.pos, clusters=clusters)
    for step in range(5):
        _, F = _oracle_forces(case, terms, x)
        x, v = M.langevin_step(x, v, F, inv_m, 300.0, 2.0, 0.001, 9, step, clusters)
    sim.step(5)
    s = sim.getState(getPositions=True, getVelocities=True)
    assert np.abs(s.getPositions() - x).max() < 1e-6
    assert np.abs(s.getVelocities() - v).max() < 5e-3


def test_constraints_hold_and_runs_are_reproducible():
    case, terms = _case(seed=9)
    runs = []
    for seed in (21, 21, 22):
        sim, _ = _sim(case, terms, seed=seed)
        sim.setVelocitiesToTemperature(300.0, 1)
        sim.step(40)
        runs.append(sim.getState(getPositions=True).getPositions())
    assert np.array_equal(runs[0], runs[1])  # same seed: the same trajectory, bit for bit
    assert not np.array_equal(runs[0], runs[2])
    x = runs[0]
    for i, j, d in terms.constraints:
        assert abs(np.linalg.norm(x[i] - x[j]) - d) < 1e-8


def test_thermostat_reaches_temperature():
    case, terms = _case(seed=10)
    sim, _ = _sim(case, terms, T=300.0, gamma=10.0, dt=0.002, seed=4)
    sim.setVelocitiesToTemperature(300.0, 2)
    sim.step(300)
    temps = []
    for _ in range(40):
        sim.step(10)
        temps.append(sim.temperatures(sim.getState(getEnergy=True).getKineticEnergy() * np.ones(1))[0])
    assert abs(np.mean(temps) - 300.0) < 25.0, np.mean(temps)


def test_verlet_energy_drift_is_small():
    case, terms = _case(seed=11)
    sim, integ = _sim(case, terms, T=300.0, gamma=10.0, dt=0.001, seed=6)
    sim.setVelocitiesToTemperature(300.0, 5)
    sim.step(400)  # relax the built structure under the thermostat
    integ.setFriction(0.0)
    integ.setTemperature(0.0)
    tot = []
    for _ in range(30):
        sim.step(10)
        st = sim.getState(getEnergy=True)
        tot.append(st.getPotentialEnergy() + st.getKineticEnergy())
    tot = np.array(tot)
    ke = sim.getState(getEnergy=True).getKineticEnergy()
    # no thermostat: the total energy wanders by a small fraction of the kinetic energy
    assert np.abs(tot - tot[0]).max() < 0.02 * ke, (np.abs(tot - tot[0]).max(), ke)


def test_batched_replicas_match_oracle_steps():
    # two replicas of different ATM parameters in one batch: each takes the
    # oracle step from its own forces with its own noise stream (replica index)
    cases = [_case(seed=s) for s in (12, 13)]
    cases[1][0].params = S.default_params(0.1, 0.5, 0.1, 30.0, 0.0, 200.0, 100.0, 0.0625, 1.0)
    systems = [atm.md_system_from_case(c, t)[0] for c, t in cases]
    integ = atm.LangevinIntegrator(300.0, 1.0, 0.002)
    integ.setRandomNumberSeed(77)
    rs = atm.ReplicaSimulation(systems, integ, 0)
    rs.setPositions(np.concatenate([c.pos for c, _ in cases]))
    rs.setVelocitiesToTemperature(300.0, 31)
    s0 = rs.getState(getVelocities=True, getForces=True, getEnergy=True)
    rs.step(1)
    s1 = rs.getState(getPositions=True, getVelocities=True)
    for k, (c, t) in enumerate(cases):
        lo, hi = rs.offsets[k], rs.offsets[k + 1]
        inv_m = 1.0 / t.masses
        clusters = M.constraint_clusters(t.constraints, c.n)
        v0 = M.velocities_at(300.0, inv_m, 31, replica=k, x=c.pos, clusters=clusters)
        np.testing.assert_allclose(s0.getVelocities()[lo:hi], v0, rtol=0, atol=1e-6)
        E_ref, F_ref = _oracle_forces(c, t, c.pos)
        F = s0.getForces()[lo:hi]
        assert np.sqrt(((F - F_ref) ** 2).sum() / (F_ref ** 2).sum()) <= 1e-4
        x1, v1 = M.langevin_step(c.pos, s0.getVelocities()[lo:hi], F, inv_m, 300.0, 1.0, 0.002, 77, 0, clusters,
                                 replica=k)
        np.testing.assert_allclose(s1.getPositions()[lo:hi], x1, rtol=0, atol=1e-10)
        np.testing.assert_allclose(s1.getVelocities()[lo:hi], v1, rtol=0, atol=1e-7)
    info = rs.info()
    assert info["steps"] == 1 and len(info["dof"]) == 2
    assert info["dof"][0] == 3 * cases[0][0].n - len(cases[0][1].constraints)


def test_batch_and_single_agree_without_noise():
    # T = 0: the batch and a single run of replica 0 follow the same deterministic path
    c, t = _case(seed=17)
    c2, t2 = _case(seed=18)
    integ = atm.LangevinIntegrator(0.0, 1.0, 0.002)
    rs = atm.ReplicaSimulation([atm.md_system_from_case(c, t)[0], atm.md_system_from_case(c2, t2)[0]], integ, 0)
    rs.setPositions(np.concatenate([c.pos, c2.pos]))
    rs.step(5)
    xb = rs.getState(getPositions=True).getPositions()
    for k, (cc, tt) in enumerate(((c, t), (c2, t2))):
        sim, _ = _sim(cc, tt, T=0.0)
        sim.step(5)
        x = sim.getState(getPositions=True).getPositions()
        assert np.abs(xb[rs.offsets[k]:rs.offsets[k + 1]] - x).max() < 1e-8


def test_reorder_keeps_the_trajectory():
    case, terms = _case(seed=14)
    out = []
    # lists built at every step in both runs: the re-sort is what differs
    for props in ({"ReorderInterval": 0, "ListSkin": 0}, {"ReorderInterval": 3, "ListSkin": 0}):
        sim, _ = _sim(case, terms, seed=8, props=props)
        sim.setVelocitiesToTemperature(300.0, 4)
        sim.step(10)
        out.append((sim.getState(getPositions=True).getPositions(), sim.info()["reorders"]))
    assert out[1][1] >= 2
    assert np.abs(out[0][0] - out[1][0]).max() < 1e-8


def test_parameters_per_replica_change_forces():
    case, terms = _case(seed=15)
    sim, _ = _sim(case, terms)
    f1 = sim.getState(getForces=True).getForces()
    sim.setParameter(0, "ATMLambda2", 0.9)
    sim.setParameter(0, "ATMLambda1", 0.9)
    f2 = sim.getState(getForces=True).getForces()
    case.params = case.params.copy()
    case.params[0], case.params[1] = 0.9, 0.9
    _, F_ref = _oracle_forces(case, terms, case.pos)
    assert np.sqrt(((f2 - F_ref) ** 2).sum() / (F_ref ** 2).sum()) <= 1e-4
    assert not np.allclose(f1, f2)


def test_errors_are_reported():
    case, terms = _case(seed=16)
    sys_, _, _ = atm.md_system_from_case(case, terms)
    integ = atm.LangevinIntegrator(300.0, 1.0, 0.002)
    sim = atm.Simulation(sys_, integ, 0)
    with pytest.raises(atm.ATMError) as e:
        sim.step(1)  # no positions yet
    assert e.value.code == 3
    with pytest.raises(atm.ATMError):
        sim.setPositions(np.zeros((5, 3)))
    # a cluster of 5 constrained particles is outside the SHAKE clusters
    sys2, _, _ = atm.md_system_from_case(case, terms)
    for j in range(1, 5):
        sys2.addConstraint(case.ligands[0][0], case.ligands[0][j], 0.15 * j)
    with pytest.raises(atm.ATMError) as e:
        atm.Simulation(sys2, atm.LangevinIntegrator(300.0, 1.0, 0.002), 0)
    assert e.value.code == 5


def test_recording_streams_results_and_energy_matrices():
    cases = [_case(seed=s) for s in (19, 20)]
    cases[1][0].params = S.default_params(0.2, 0.4, 0.1, 25.0, 0.0, 200.0, 100.0, 0.0625, 1.0)
    systems = [atm.md_system_from_case(c, t)[0] for c, t in cases]
    integ = atm.LangevinIntegrator(300.0, 1.0, 0.002)
    integ.setRandomNumberSeed(5)
    rs = atm.ReplicaSimulation(systems, integ, 0)
    rs.setPositions(np.concatenate([c.pos for c, _ in cases]))
    rs.setVelocitiesToTemperature(300.0, 3)
    rs.setRecording(2, capacity=8)
    s0 = rs.getState(getEnergy=True)
    rs.step(6)
    rec = rs.getRecords()
    assert list(rec["steps"]) == [0, 2, 4]
    # the first record is the evaluation the state at step 0 reported
    res0 = np.array([[r[k] for k in atm.RES_KEYS] for r in s0.getResults()])
    np.testing.assert_array_equal(rec["results"][0], res0)
    beta = 1.0 / (M.KB * 300.0)
    iE1, iE2 = atm.RES_KEYS.index("E1"), atm.RES_KEYS.index("E2")
    for k in range(3):
        R = rec["results"][k]
        for r in range(2):
            for q in range(2):
                ref = beta * O.atm_merge(R[r, iE1], R[r, iE2], cases[q][0].params)["energy"]
                assert abs(rec["matrices"][k][r, q] - ref) <= 1e-9 * max(1.0, abs(ref))
    assert len(rs.getRecords()["steps"]) == 0  # the ring was emptied
    # a full ring keeps the newest records
    rs.setRecording(1, capacity=2)
    rs.step(5)
    assert list(rs.getRecords()["steps"]) == [9, 10]
