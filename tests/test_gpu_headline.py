"""Parity of the benchmarked workloads with the FP64 oracle, replica by replica.

- 22 replicas of the 23,558-atom PME box on the 22-state softplus schedule
  (alpha 0.1 /(kJ/mol), u0 110 kJ/mol): the batch ``bench.py`` times, in the
  difference mode it times, every replica checked; and the plain single-replica
  drop-in (two full inner evaluations) of its first replica;
- the full 22 x 22 reduced-energy matrix of that batch against the oracle's merge
  of every replica's (E1, E2) under every replica's parameters;
- 22 replicas of the 60,000-atom two-ligand RBFE box on the same schedule
  (three replicas checked: first, middle, last).

Tolerances (the targets of the path): |u - u_oracle| <= 0.01 kJ/mol, force RMS
relative error <= 1e-4; total energies within 2e-6 of the summed magnitudes of
their terms (FP32 pair arithmetic).  Semantics per replica: the merge of
ReferenceATMMetaForceKernels.cpp:56-113.
"""
import os

import numpy as np
import pytest

import atmmetaforce as atm
import oracle as O
from atmmetaforce import synthetic as S

pytestmark = pytest.mark.gpu

U_TOL = 0.01
F_TOL = 1e-4
BETA = 1.0 / (0.0083144626 * 300.0)


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


def force_rel(F, G):
    return float(np.sqrt(((F - G) ** 2).sum() / (G ** 2).sum()))


def energy_tol(spec, pos):
    _, _, T = O.nonbonded(spec, pos, forces=False)
    return 2e-6 * (sum(abs(v) for v in T.values()) + 1.0)


@pytest.fixture(scope="module")
def headline():
    cases = S.abfe_pme_23558_x22()
    b = atm.ReplicaBatch([atm.system_from_case(c)[0] for c in cases], 0, {"DifferencePath": 1})
    E, F, res = b.evaluate(np.concatenate([c.pos for c in cases]))
    refs = [O.atm_eval(c.spec, c.pos, c.displ, c.params) for c in cases]
    M = b.energyMatrix(beta=BETA)
    return cases, b, E, F, res, refs, M


def test_headline_batch_every_replica(headline):
    cases, b, E, F, res, refs, M = headline
    assert b.stats()["max_row"] > 0
    du, fr = [], []
    for k, (c, ref) in enumerate(zip(cases, refs)):
        assert res[k]["status"] == 0
        du.append(abs(res[k]["pert"] - ref["usc"]))
        fr.append(force_rel(F[b.offsets[k]:b.offsets[k + 1]], ref["forces"]))
        # the FP64 merge of the record's own energies is the oracle's merge (sp moves
        # with u; u itself is held to its tolerance below)
        m = O.atm_merge(res[k]["E1"], res[k]["E2"], c.params)
        assert abs(res[k]["sp"] - m["sp"]) <= 1e-9 * max(1.0, abs(m["sp"])), k
        assert abs(res[k]["W"] - m["W"]) <= 1e-9 * max(1.0, abs(m["W"])), k
        assert abs(E[k] - ref["energy"]) <= energy_tol(c.spec, c.pos), k
    print(f"22 x 23,558: max |du| {max(du):.2e} kJ/mol, max force rms rel {max(fr):.2e}")
    assert max(du) <= U_TOL, du
    assert max(fr) <= F_TOL, fr


def test_headline_energy_matrix(headline):
    cases, b, E, F, res, refs, M = headline
    R = len(cases)
    assert M.shape == (R, R)
    for r in range(R):
        tol_abs = BETA * (energy_tol(cases[r].spec, cases[r].pos) + U_TOL)
        # the oracle's merge of replica r's energies at x and x + d under state s's parameters
        row = np.array([O.atm_merge(refs[r]["E1"], refs[r]["E2"], cases[s].params)["energy"] for s in range(R)])
        assert np.all(np.abs(M[r] - BETA * row) <= tol_abs), r
        # differences along a row drop the common state-1 energy: they carry only
        # W(u) and must agree to the u tolerance (|dW/du| <= 1 on this schedule)
        assert np.all(np.abs((M[r] - M[r, 0]) - BETA * (row - row[0])) <= 2 * BETA * U_TOL), r


def test_headline_batch_through_the_fused_kernel(headline):
    """The same batch with the lists and pair tiles in one persistent kernel
    (FusedTiles=1, which the autotuner may choose): every replica against the
    oracle, and against the two-kernel path (FP32 pair sums in another order)."""
    cases, b, E, F, res, refs, M = headline
    fb = atm.ReplicaBatch([atm.system_from_case(c)[0] for c in cases], 0, {"DifferencePath": 1, "FusedTiles": 1})
    E2, F2, res2 = fb.evaluate(np.concatenate([c.pos for c in cases]))
    assert force_rel(F2, F) <= 1e-5
    du = []
    for k, (c, ref) in enumerate(zip(cases, refs)):
        assert res2[k]["status"] == 0
        du.append(abs(res2[k]["pert"] - ref["usc"]))
        assert force_rel(F2[fb.offsets[k]:fb.offsets[k + 1]], ref["forces"]) <= F_TOL, k
        assert abs(E2[k] - ref["energy"]) <= energy_tol(c.spec, c.pos), k
    assert max(du) <= U_TOL, du


def test_plain_single_replica_at_bench_settings(headline):
    cases, b, E, F, res, refs, M = headline
    c = cases[0]
    pb = atm.ReplicaBatch([atm.system_from_case(c)[0]], 0, {"DifferencePath": 0})
    E1, F1, r1 = pb.evaluate(c.pos)
    assert abs(r1[0]["pert"] - refs[0]["usc"]) <= U_TOL
    assert force_rel(F1, refs[0]["forces"]) <= F_TOL
    assert abs(E1[0] - refs[0]["energy"]) <= energy_tol(c.spec, c.pos)


def test_rbfe_batch_of_22():
    cases = []
    for r in range(22):
        l1, l2 = S.SCHEDULE_22[r]
        c = S.rbfe_pme_60000(seed=400 + r)
        c.params = S.default_params(l1, l2, 0.1, 110.0, 0.0, 200.0, 100.0, 0.0625, 1.0)
        cases.append(c)
    b = atm.ReplicaBatch([atm.system_from_case(c)[0] for c in cases], 0, {"DifferencePath": 1})
    E, F, res = b.evaluate(np.concatenate([c.pos for c in cases]))
    for k in (0, 11, 21):
        c = cases[k]
        ref = O.atm_eval(c.spec, c.pos, c.displ, c.params)
        assert res[k]["status"] == 0
        assert abs(res[k]["pert"] - ref["usc"]) <= U_TOL, k
        assert force_rel(F[b.offsets[k]:b.offsets[k + 1]], ref["forces"]) <= F_TOL, k
        assert abs(E[k] - ref["energy"]) <= energy_tol(c.spec, c.pos), k
        # TI derivatives of the record against the oracle's merge: both move with
        # usc by at most |d/dusc| <= 1, so they carry the u tolerance
        g = O.softplus_param_grad(ref["usc"], c.params)
        assert abs(res[k]["dW_dlambda1"] - g[0]) <= U_TOL, k
        assert abs(res[k]["dW_dlambda2"] - g[1]) <= 2 * U_TOL, k
