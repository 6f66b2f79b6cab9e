"""Pair lists kept across evaluations (the neighbour-list skin) on the GPU.

With a skin, the lists are built at the cutoff plus the skin and kept until an
atom has moved more than half the skin since their build; the GPU checks that
at every evaluation.  Results must not depend on whether the lists were kept:
against the FP64 oracle, u within 0.01 kJ/mol and force RMS relative error
<= 1e-4; against the same batch without a skin, forces within 1e-5 relative
(FP32 pair sums in another order).  In MD, steps are enqueued without a host
synchronisation per step and the list status is read every CheckInterval steps;
a run whose checks send it back to a snapshot must follow the same trajectory.
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


@pytest.mark.parametrize("fused", [0, 1], ids=["two-kernels", "fused"])
@pytest.mark.parametrize("method,diff", [(S.PME, 1), (S.PME, 0), (S.CUTOFF_PERIODIC, 1)],
                         ids=["pme-difference", "pme-two-states", "rf-difference"])
def test_kept_lists_give_the_results_of_fresh_ones(method, diff, fused):
    case = S.water_ligand_box(6000, 3.9, [18], [(1.9, 1.8, 2.0)], method, 0.9, seed=91,
                              params=S.default_params(0.3, 0.6, 0.1, 20.0, 0.0))
    sys_ = atm.system_from_case(case)[0]
    kept = atm.ReplicaBatch([sys_], 0, {"DifferencePath": diff, "ListSkin": 0.1, "FusedTiles": fused})
    fresh = atm.ReplicaBatch([atm.system_from_case(case)[0]], 0, {"DifferencePath": diff})
    rng = np.random.default_rng(3)
    p0 = case.pos
    p1 = p0 + rng.uniform(-0.02, 0.02, p0.shape)  # every atom within 0.035 nm < skin / 2
    p2 = p1.copy()
    p2[5] += (0.06, 0.0, 0.0)                      # one atom beyond skin / 2
    # builds added by each evaluation (the first one may also have grown capacities)
    expect_new_builds = [None, 0, 1]
    prev = prev0 = None
    for k, pos in enumerate((p0, p1, p2)):
        E, F, res = kept.evaluate(pos)
        E0, F0, res0 = fresh.evaluate(pos)
        info, info0 = kept.listInfo(), fresh.listInfo()
        assert info["skin"] == 0.1
        if prev is not None:
            assert info["evaluations"] - prev["evaluations"] == 1
            assert info["builds"] - prev["builds"] == expect_new_builds[k], (k, prev, info)
            assert info0["builds"] - prev0["builds"] == 1  # no skin: built every time
        prev, prev0 = info, info0
        assert force_rel(F, F0) <= 1e-5
        assert abs(res[0]["pert"] - res0[0]["pert"]) <= 1e-3
        ref = O.atm_eval(case.spec, pos, case.displ, case.params)
        assert abs(res[0]["pert"] - ref["usc"]) <= U_TOL
        assert force_rel(F, ref["forces"]) <= F_TOL


def test_skin_larger_than_the_box_allows_is_refused():
    case = S.water_ligand_box(1500, 2.5, [10], [(1.2, 1.2, 1.2)], S.PME, 0.9, seed=92)
    with pytest.raises(atm.ATMError):
        atm.ReplicaBatch([atm.system_from_case(case)[0]], 0, {"ListSkin": 0.4})  # 2 (0.9 + 0.4) > 2.5


def _md(props, steps, seed=5):
    case = S.abfe_pme_small(4000, 14, seed=93)
    case.params = S.default_params(0.3, 0.6, 0.1, 20.0, 0.0, 200.0, 100.0, 0.0625, 1.0)
    terms, pos = S.md_terms_ligand_centroid(case)
    sys_, _, _ = atm.md_system_from_case(case, terms)
    integ = atm.LangevinIntegrator(300.0, 50.0, 0.002)
    integ.setRandomNumberSeed(seed)
    sim = atm.Simulation(sys_, integ, 0, props)
    sim.setPositions(pos)
    sim.setVelocitiesToTemperature(300.0, 11)
    sim.step(steps)
    return sim


def test_md_with_kept_lists_follows_the_rebuilt_trajectory():
    a = _md({"ListSkin": 0.0, "CheckInterval": 1}, 60)
    b = _md({"ListSkin": 0.1, "CheckInterval": 10}, 60)
    c = _md({"ListSkin": 0.1, "CheckInterval": 10, "FusedTiles": 1}, 60)  # lists and tiles in one kernel
    xa = a.getState(getPositions=True).getPositions()
    xb = b.getState(getPositions=True).getPositions()
    xc = c.getState(getPositions=True).getPositions()
    assert np.abs(xa - xb).max() <= 1e-4
    assert np.abs(xa - xc).max() <= 1e-4
    assert c.listInfo()["builds"] < c.listInfo()["evaluations"]
    ib = b.listInfo()
    assert ib["builds"] < ib["evaluations"]  # the lists were kept between builds
    assert a.listInfo()["builds"] == a.listInfo()["evaluations"]


def test_md_spreading_per_atom_follows_the_same_trajectory():
    """Spreading per atom (SpreadBrick=0) adds the same integer stencil
    contributions to the charge grids as the bricks: an MD run with it follows the
    trajectory of bricks of 16 bit for bit."""
    a = _md({"ListSkin": 0.1, "SpreadBrick": 16}, 30)
    b = _md({"ListSkin": 0.1, "SpreadBrick": 0}, 30)
    xa = a.getState(getPositions=True).getPositions()
    xb = b.getState(getPositions=True).getPositions()
    assert np.array_equal(xa, xb)


def test_md_check_that_reports_an_overflow_redoes_the_steps():
    """The host-side fake makes the second list check report an overflow: the
    state goes back to the snapshot of the first check and the steps run again,
    with lists built anew, along the same trajectory."""
    a = _md({"ListSkin": 0.1, "CheckInterval": 10}, 40)
    b = _md({"ListSkin": 0.1, "CheckInterval": 10, "TestFailListCheck": 2}, 40)
    assert b.listInfo()["redos"] == 1 and a.listInfo()["redos"] == 0
    assert b.info()["steps"] == a.info()["steps"] == 40
    xa = a.getState(getPositions=True).getPositions()
    xb = b.getState(getPositions=True).getPositions()
    assert np.abs(xa - xb).max() <= 1e-4


def test_md_autotune_reports_the_skin_and_keeps_the_state():
    case = S.abfe_pme_small(4000, 14, seed=94)
    terms, pos = S.md_terms_ligand_centroid(case)
    sys_, _, _ = atm.md_system_from_case(case, terms)
    integ = atm.LangevinIntegrator(300.0, 1.0, 0.002)
    sim = atm.Simulation(sys_, integ, 0)
    sim.setPositions(pos)
    sim.setVelocitiesToTemperature(300.0, 3)
    v0 = sim.getState(getVelocities=True).getVelocities()
    report = sim.autotune(trials=8)
    assert "list skin" in report and "chosen: list skin" in report
    s = sim.getState(getPositions=True, getVelocities=True)
    assert np.array_equal(s.getPositions(), pos) and np.array_equal(s.getVelocities(), v0)
    assert sim.info()["steps"] == 0
    chosen = float(report.strip().splitlines()[-1].split("list skin")[1].split("nm")[0])
    assert sim.listInfo()["skin"] == chosen
