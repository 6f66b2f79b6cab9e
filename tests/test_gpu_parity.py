"""Parity of the CUDA path with the FP64 oracle, through the C ABI.

Tolerances (the targets of the path): perturbation energy u within 0.01 kJ/mol,
force RMS relative error <= 1e-4.  Total energies, which the reference gives in
double precision, are compared with a relative tolerance of 2e-6 of the sum of
the magnitudes of the energy terms (FP32 pair arithmetic).
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


def energy_tol(spec, pos):
    _, _, T = O.nonbonded(spec, pos, forces=False)
    return 2e-6 * (sum(abs(v) for v in T.values()) + 1.0)


def run_context(case, diff, groups=(2,), fused=0):
    sys_, nb, f = atm.system_from_case(case)
    ctx = atm.Context(sys_, 0, {"DifferencePath": int(diff), "FusedTiles": int(fused)})
    ctx.setPositions(case.pos)
    st = ctx.getState(getEnergy=True, getForces=True, groups=set(groups))
    return ctx, f, st


def check_case(case, diff, fused=0):
    ctx, f, st = run_context(case, diff, fused=fused)
    ref = O.atm_eval(case.spec, case.pos, case.displ, case.params)
    u = f.getPerturbationEnergy(ctx)
    assert abs(u - ref["usc"]) <= U_TOL, (u, ref["usc"])
    assert force_rel(st.getForces(), ref["forces"]) <= F_TOL
    tol = energy_tol(case.spec, case.pos)
    assert abs(st.getPotentialEnergy() - ref["energy"]) <= tol, (st.getPotentialEnergy(), ref["energy"], tol)
    r = st.getResults()
    assert r["status"] == 0
    # sp is the FP64 merge of the record's own energies, and it moves with u: it is
    # held to the u tolerance times its slope dsp/du (central difference of the merge)
    m = O.atm_merge(r["E1"], r["E2"], case.params)
    assert abs(r["sp"] - m["sp"]) <= 1e-9 * max(1.0, abs(m["sp"]))
    h = 1e-3
    slope = abs(O.atm_merge(ref["E1"], ref["E2"] + h, case.params)["sp"] -
                O.atm_merge(ref["E1"], ref["E2"] - h, case.params)["sp"]) / (2 * h)
    assert abs(r["sp"] - ref["sp"]) <= 2 * slope * U_TOL + 1e-9, (r["sp"], ref["sp"], slope)
    return ctx, f, st, ref


@pytest.mark.parametrize("diff", [0, 1], ids=["two-states", "difference"])
def test_reaction_field_2394(diff):
    check_case(S.abfe_rf_2394(0), diff)


@pytest.mark.parametrize("diff", [0, 1], ids=["two-states", "difference"])
@pytest.mark.parametrize("method", [S.NOCUTOFF, S.CUTOFF_NONPERIODIC], ids=["no-cutoff", "cutoff-nonperiodic"])
def test_nonperiodic_methods(method, diff):
    """NoCutoff (plain Coulomb + LJ over every pair) and CutoffNonPeriodic
    (reaction field within the cutoff), no periodic images: the inner
    NonbondedForce the reference re-evaluates may use either."""
    c = S.water_ligand_box(2394, 3.0, [24], [(1.5, 1.5, 1.5)], method, 0.9, seed=5,
                           params=S.default_params(0.4, 0.6, 0.05, 10.0, 0.0))
    check_case(c, diff)


TRICLINIC = {"moderate": ((4.0, 3.8, 3.7), (1.2, -1.0, 0.9)), "skewed": ((4.0, 3.8, 3.7), (1.9, 1.8, -1.8))}


@pytest.mark.parametrize("diff", [0, 1], ids=["two-states", "difference"])
@pytest.mark.parametrize("shape", list(TRICLINIC), ids=list(TRICLINIC))
@pytest.mark.parametrize("method", [S.PME, S.CUTOFF_PERIODIC], ids=["pme", "reaction-field"])
def test_triclinic_boxes(method, shape, diff):
    """OpenMM's reduced triclinic boxes (System::setDefaultPeriodicBoxVectors):
    minimum images c, then b, then a; PME in fractional coordinates."""
    box, tilt = TRICLINIC[shape]
    c = S.triclinic_water_ligand_box(5500, box, tilt, [16], [(1.6, 1.5, 1.4)], method, 0.9, seed=13,
                                     params=S.default_params(0.3, 0.6, 0.1, 20.0, 0.0))
    check_case(c, diff)


@pytest.mark.parametrize("method", [S.PME, S.CUTOFF_PERIODIC, S.NOCUTOFF], ids=["pme", "reaction-field", "no-cutoff"])
@pytest.mark.parametrize("diff", [0, 1], ids=["two-states", "difference"])
def test_fused_lists_and_tiles_kernel(diff, method):
    """FusedTiles=1: one persistent kernel builds each row's lists and evaluates
    its tiles, in a triclinic box for the periodic methods."""
    if method == S.NOCUTOFF:
        c = S.water_ligand_box(1500, 2.5, [10], [(1.2, 1.1, 1.0)], method, 0.9, seed=17,
                               params=S.default_params(0.3, 0.6, 0.1, 20.0, 0.0))
    else:
        box, tilt = TRICLINIC["skewed"]
        c = S.triclinic_water_ligand_box(5500, box, tilt, [16], [(1.6, 1.5, 1.4)], method, 0.9, seed=18,
                                         params=S.default_params(0.3, 0.6, 0.1, 20.0, 0.0))
    check_case(c, diff, fused=1)


@pytest.mark.parametrize("diff", [0, 1], ids=["two-states", "difference"])
def test_small_triclinic_box_with_per_pair_images(diff):
    """A box so small against the cutoff that pairs take their own images (the
    list building searches the 125 images around the blocks' minimum image)."""
    c = S.triclinic_water_ligand_box(1500, (2.6, 2.5, 2.4), (0.8, -0.7, 0.6), [10], [(1.2, 1.1, 1.0)], S.PME, 0.9,
                                     seed=14, params=S.default_params(0.3, 0.6, 0.1, 20.0, 0.0))
    check_case(c, diff)


def test_batch_of_triclinic_and_orthorhombic_replicas():
    cases = [S.triclinic_water_ligand_box(5500, (4.0, 3.8, 3.7), (1.2, -1.0, 0.9), [16], [(1.6, 1.5, 1.4)], S.PME,
                                          0.9, seed=15),
             S.water_ligand_box(5000, 3.7, [16], [(1.6, 1.5, 1.4)], S.PME, 0.9, seed=16)]
    b = atm.ReplicaBatch([atm.system_from_case(c)[0] for c in cases], 0)
    E, F, res = b.evaluate(np.concatenate([c.pos for c in cases]))
    for k, c in enumerate(cases):
        ref = O.atm_eval(c.spec, c.pos, c.displ, c.params)
        assert abs(res[k]["pert"] - ref["usc"]) <= U_TOL, k
        assert force_rel(F[b.offsets[k]:b.offsets[k + 1]], ref["forces"]) <= F_TOL, k


@pytest.mark.parametrize("diff", [0, 1], ids=["two-states", "difference"])
def test_pme_small(diff):
    c = S.water_ligand_box(3000, 3.1, [16], [(1.4, 1.3, 1.5)], S.PME, 0.9, seed=11,
                           params=S.default_params(0.2, 0.7, 0.1, 30.0, 2.0))
    check_case(c, diff)


@pytest.mark.parametrize("diff", [0, 1], ids=["two-states", "difference"])
def test_pme_23558(diff):
    check_case(S.abfe_pme_23558(1), diff)


@pytest.mark.parametrize("diff", [0, 1], ids=["two-states", "difference"])
def test_rbfe_two_ligands_60000(diff):
    """Relative swap: ligand A displaced +(2.5,2.5,2.5), ligand B -(2.5,2.5,2.5);
    the difference path must also count the A x B pairs, which move relative to
    each other."""
    check_case(S.rbfe_pme_60000(), diff)


def test_page_locked_buffers_give_the_same_results():
    """Page-locked positions are read without a staging copy and page-locked
    force buffers are written by the output kernel over the host link: the
    results must be those of ordinary host buffers, bit for bit."""
    import torch

    cases = [S.water_ligand_box(3000, 3.1, [16], [(1.4, 1.3, 1.5)], S.PME, 0.9, seed=31 + k) for k in range(3)]
    b = atm.ReplicaBatch([atm.system_from_case(c)[0] for c in cases], 0)
    pos = np.concatenate([c.pos for c in cases])
    E0, F0, r0 = b.evaluate(pos, as_array=True)
    M0 = b.energyMatrix(beta=0.4)
    pos_pin = torch.from_numpy(pos).pin_memory().numpy()
    F_pin = torch.full(pos.shape, float("nan"), dtype=torch.float64).pin_memory().numpy()
    for _ in range(2):
        E1, F1, r1 = b.evaluate(pos_pin, out=F_pin, as_array=True)
        assert np.array_equal(F1, F0) and np.array_equal(E1, E0) and np.array_equal(r1, r0)
        assert np.array_equal(b.energyMatrix(beta=0.4), M0)
    # and ordinary buffers again afterwards (the page-locked target is not kept)
    E2, F2, r2 = b.evaluate(pos, as_array=True)
    assert np.array_equal(F2, F0) and np.array_equal(F_pin, F0)
    for k, c in enumerate(cases):
        ref = O.atm_eval(c.spec, c.pos, c.displ, c.params)
        assert abs(r1[k][atm.RES_KEYS.index("pert")] - ref["usc"]) <= U_TOL
        assert force_rel(F1[b.offsets[k]:b.offsets[k + 1]], ref["forces"]) <= F_TOL


def test_mixed_batch_of_eight_uneven_boxes():
    cases = S.mixed_batch_8()
    b = atm.ReplicaBatch([atm.system_from_case(c)[0] for c in cases], 0)
    E, F, res = b.evaluate(np.concatenate([c.pos for c in cases]))
    for k, c in enumerate(cases):
        ref = O.atm_eval(c.spec, c.pos, c.displ, c.params)
        assert abs(res[k]["pert"] - ref["usc"]) <= U_TOL, k
        assert force_rel(F[b.offsets[k]:b.offsets[k + 1]], ref["forces"]) <= F_TOL, k


def test_deterministic_bitwise():
    c = S.water_ligand_box(3000, 3.1, [16], [(1.4, 1.3, 1.5)], S.PME, 0.9, seed=12)
    sys_, nb, f = atm.system_from_case(c)
    ctx = atm.Context(sys_, 0, {"DifferencePath": 1})
    ctx.setPositions(c.pos)
    a = ctx.getState(getEnergy=True, getForces=True, groups={2})
    ctx.setPositions(c.pos)  # forces a second evaluation
    b = ctx.getState(getEnergy=True, getForces=True, groups={2})
    assert np.array_equal(a.getForces(), b.getForces())
    assert a.getPotentialEnergy() == b.getPotentialEnergy()


@pytest.mark.parametrize("diff", [0, 1], ids=["two-states", "difference"])
def test_spreading_by_owner_gives_the_same_bits(diff):
    """PME spreading by owner brick (each atom spread once, by the brick holding
    its stencil base; bricks summed into int32 grids by atomics) and spreading per
    atom (SpreadBrick=0: each atom's stencil added straight into the grid by
    atomics) add the same integer stencil contributions to every grid point as
    spreading by every brick a stencil touches, so grids and results must be the
    same bits.  Grids of several sizes, a triclinic box, and both grids of the
    difference path (the moving atoms' update grid is mostly empty bricks)."""
    cases = [S.water_ligand_box(3000, 3.1, [16], [(1.4, 1.3, 1.5)], S.PME, 0.9, seed=41),
             S.water_ligand_box(9000, 4.5, [24], [(1.6, -1.5, 1.4)], S.PME, 0.9, seed=42),
             S.triclinic_water_ligand_box(5500, (4.0, 3.8, 3.7), (1.2, -1.0, 0.9), [16], [(1.6, 1.5, 1.4)], S.PME,
                                          0.9, seed=43)]
    systems = [atm.system_from_case(c)[0] for c in cases]
    pos = np.concatenate([c.pos for c in cases])
    out = {}
    modes = {"touching bricks": {"SpreadByOwner": 0}, "owner bricks": {"SpreadByOwner": 1},
             "per atom": {"SpreadBrick": 0}, "owner bricks of 12": {"SpreadBrick": 12}}
    for name, props in modes.items():
        b = atm.ReplicaBatch(systems, 0, {"DifferencePath": diff, **props})
        out[name] = b.evaluate(pos, as_array=True), b.energyMatrix(beta=0.4), b.offsets
    (E0, F0, r0), M0, _ = out["touching bricks"]
    for name in modes:
        (E1, F1, r1), M1, offs = out[name]
        assert np.array_equal(F0, F1) and np.array_equal(E0, E1) and np.array_equal(r0, r1), name
        assert np.array_equal(M0, M1), name
    for k, c in enumerate(cases):
        ref = O.atm_eval(c.spec, c.pos, c.displ, c.params)
        assert abs(r1[k][atm.RES_KEYS.index("pert")] - ref["usc"]) <= U_TOL, k
        assert force_rel(F1[offs[k]:offs[k + 1]], ref["forces"]) <= F_TOL, k


@pytest.mark.parametrize("diff", [0, 1], ids=["two-states", "difference"])
def test_displaced_ligand_overlapping_a_water(diff):
    """A ligand atom whose displaced position lies 0.05 nm from a water oxygen:
    u reaches about 4e9 kJ/mol, beyond 2^31, in the range the soft-core exists to
    absorb (an MD step can produce it).  The energies must be summed without a
    range limit: u within 1e-4 relative of the oracle (a range limit shows as an
    error of tens of percent; FP32 pair arithmetic gives about 3e-5 here, where
    r^-12 multiplies the relative error of the hardware reciprocal square root
    twelvefold), the soft-core perturbation energy within the usual tolerance.  (The pair's force, about 1e12 kJ/mol/nm,
    is beyond the range of the fixed-point force sums, 2^31 kJ/mol/nm; the merge
    weights it by sp, about 1e-10 here, and it is not compared.)"""
    c = S.water_ligand_box(3000, 3.1, [16], [(1.4, 1.3, 1.5)], S.PME, 0.9, seed=44)
    lig = np.nonzero(np.abs(c.displ).sum(axis=1) > 0)[0]
    k = lig[len(lig) // 2]
    c.pos[k] = c.pos[0] - c.displ[k] + np.array([0.05, 0.0, 0.0])  # atom 0 is a water oxygen
    ref = O.atm_eval(c.spec, c.pos, c.displ, c.params)
    assert ref["u"] > 2.0 ** 31
    b = atm.ReplicaBatch([atm.system_from_case(c)[0]], 0, {"DifferencePath": diff})
    E, F, r = b.evaluate(c.pos)
    assert abs(r[0]["u"] - ref["u"]) <= 1e-4 * abs(ref["u"])
    assert abs(r[0]["pert"] - ref["usc"]) <= U_TOL


def test_batch_mixed_sizes_vs_oracle_and_matrix():
    cases = [S.abfe_pme_small(1500, 8, 21), S.abfe_pme_small(4000, 18, 22),
             S.abfe_pme_small(2500, 12, 23, displ=1.2), S.abfe_pme_small(6000, 30, 24)]
    for k, c in enumerate(cases):
        l1, l2 = S.SCHEDULE_22[5 * k]
        c.params = S.default_params(l1, l2, 0.1, 110.0 - 40 * k, 0.5 * k, 200.0, 100.0, 0.0625, 1.0 if k != 2 else -1.0)
    systems = [atm.system_from_case(c)[0] for c in cases]
    b = atm.ReplicaBatch(systems, 0)
    pos = np.concatenate([c.pos for c in cases])
    E, F, res = b.evaluate(pos)
    refs = []
    for k, c in enumerate(cases):
        ref = O.atm_eval(c.spec, c.pos, c.displ, c.params)
        refs.append(ref)
        assert abs(res[k]["pert"] - ref["usc"]) <= U_TOL
        Fk = F[b.offsets[k]:b.offsets[k + 1]]
        assert force_rel(Fk, ref["forces"]) <= F_TOL
        assert abs(E[k] - ref["energy"]) <= energy_tol(c.spec, c.pos)
    M = b.energyMatrix(beta=0.4)
    for r in range(len(cases)):
        for s in range(len(cases)):
            m = O.atm_merge(refs[r]["E1"], refs[r]["E2"], cases[s].params)
            tol = 0.4 * (energy_tol(cases[r].spec, cases[r].pos) + U_TOL)
            assert abs(M[r, s] - 0.4 * m["energy"]) <= tol


def test_autotune_keeps_parity(tmp_path, monkeypatch):
    monkeypatch.setenv("ATM_AUTOTUNE_CACHE", str(tmp_path / "tune.txt"))
    cases = [S.abfe_pme_small(3000, 14, 81), S.abfe_pme_small(3000, 14, 82)]
    b = atm.ReplicaBatch([atm.system_from_case(c)[0] for c in cases], 0)
    pos = np.concatenate([c.pos for c in cases])
    E0, F0, r0 = b.evaluate(pos)
    report = b.autotune(trials=2, use_cache=False)
    assert "chosen:" in report and report.count("ms") >= 3
    E1, F1, r1 = b.evaluate(pos)
    # every tuning gives the same bits: forces and the PME grid are integer sums
    assert np.array_equal(F1, F0)
    for k, c in enumerate(cases):
        ref = O.atm_eval(c.spec, c.pos, c.displ, c.params)
        assert abs(r1[k]["pert"] - ref["usc"]) <= U_TOL
    # a second batch of the same workload reuses the stored choice
    b2 = atm.ReplicaBatch([atm.system_from_case(c)[0] for c in cases], 0)
    b2.evaluate(pos)
    assert b2.autotune(trials=2, use_cache=True).startswith("cached")


def test_batch_matches_single_contexts():
    cases = [S.abfe_pme_small(2000, 10, 31), S.abfe_pme_small(2000, 10, 32)]
    systems = [atm.system_from_case(c)[0] for c in cases]
    b = atm.ReplicaBatch(systems, 0)
    E, F, res = b.evaluate(np.concatenate([c.pos for c in cases]))
    for k, c in enumerate(cases):
        ctx, f, st = run_context(c, 1)
        np.testing.assert_allclose(F[b.offsets[k]:b.offsets[k + 1]], st.getForces(), rtol=0, atol=1e-6)
        assert abs(res[k]["pert"] - f.getPerturbationEnergy(ctx)) < 1e-6


def test_temoa_g1_reference_pin_on_gpu():
    z = np.load(os.path.join(os.path.dirname(__file__), "golden", "temoa_g1.npz"))
    alpha, grid = S.pme_parameters(float(z["cutoff"]), float(z["ewald_tol"]), z["box_default"])
    spec = S.NonbondedSpec(charge=z["charge"], sigma=z["sigma"], epsilon=z["epsilon"], exc_i=z["exc_i"],
                           exc_j=z["exc_j"], exc_qq=z["exc_qq"], exc_sig=z["exc_sig"], exc_eps=z["exc_eps"],
                           method=S.PME, cutoff=float(z["cutoff"]), box=z["box"], alpha=alpha, grid=tuple(grid),
                           use_disp_corr=True)
    d = np.zeros_like(z["pos"])
    d[z["ligand"]] = z["displacement"]
    case = S.ATMCase(spec=spec, pos=z["pos"], displ=d, params=z["params"])
    for diff in (0, 1):
        ctx, f, st = run_context(case, diff)
        u = f.getPerturbationEnergy(ctx)
        # python/tests/test_abfe.py:148,150
        assert abs(u - float(z["expected_u"])) <= float(z["expected_u_atol"]), u
        ref = O.atm_eval(spec, z["pos"], d, z["params"])
        assert abs(u - ref["usc"]) <= U_TOL
        assert force_rel(st.getForces(), ref["forces"]) <= F_TOL


def test_parameters_softcore_direction_and_alpha_zero():
    c = S.water_ligand_box(2500, 3.0, [14], [(1.3, 1.4, 1.2)], S.PME, 0.9, seed=41)
    sys_, nb, f = atm.system_from_case(c)
    ctx = atm.Context(sys_, 0, {"DifferencePath": 1})
    ctx.setPositions(c.pos)
    E1 = O.nonbonded(c.spec, c.pos, forces=False)[0]
    E2 = O.nonbonded(c.spec, c.pos + c.displ, forces=False)[0]
    u = E2 - E1
    settings = [
        dict(ATMDirection=-1.0),
        dict(ATMDirection=1.0, ATMUbcore=u - 20.0, ATMUmax=u + 50.0, ATMAcore=0.0625),  # soft-core active
        dict(ATMAlpha=0.0, ATMLambda1=0.2, ATMLambda2=0.6),  # alpha = 0 quirk
        dict(ATMAlpha=0.3, ATMU0=u, ATMW0=3.0),
    ]
    p = c.params.copy()
    for st_ in settings:
        for k, v in st_.items():
            ctx.setParameter(k, v)
            p[S.PARAM_NAMES.index(k)] = v
        s = ctx.getState(getEnergy=True, getForces=True, groups={2})
        ref = O.atm_merge(E1, E2, p)
        assert abs(f.getPerturbationEnergy(ctx) - ref["usc"]) <= U_TOL
        assert abs(s.getResults()["sp"] - ref["sp"]) <= 1e-5
        assert abs(ctx.getParameter(list(st_)[0]) - list(st_.values())[0]) == 0


def test_group_semantics_and_nonbonded_group():
    c = S.water_ligand_box(1500, 2.5, [10], [(1.2, 1.2, 1.2)], S.PME, 0.9, seed=51)
    sys_, nb, f = atm.system_from_case(c)
    ctx = atm.Context(sys_, 0)
    ctx.setPositions(c.pos)
    # only the NonbondedForce's group: its state-1 energy and forces
    s1 = ctx.getState(getEnergy=True, getForces=True, groups={1})
    E1, F1, _ = O.nonbonded(c.spec, c.pos)
    assert abs(s1.getPotentialEnergy() - E1) <= energy_tol(c.spec, c.pos)
    assert force_rel(s1.getForces(), F1) <= F_TOL
    # the ATM group not requested: perturbation energy not refreshed (ATMMetaForceImpl.cpp:103,125)
    assert f.getPerturbationEnergy(ctx) == 0.0
    ctx.getState(getEnergy=True, groups={2})
    assert f.getPerturbationEnergy(ctx) != 0.0


def test_update_parameters_in_context_and_no_moving_atoms():
    c = S.water_ligand_box(1500, 2.5, [10], [(1.2, 1.2, 1.2)], S.PME, 0.9, seed=61)
    sys_, nb, f = atm.system_from_case(c)
    ctx = atm.Context(sys_, 0, {"DifferencePath": 1})
    ctx.setPositions(c.pos)
    ctx.getState(getEnergy=True, groups={2})
    lig = c.ligands[0]
    d2 = c.displ.copy()
    d2[lig] = (1.0, -1.1, 0.9)
    for i in lig:
        f.setParticleParameters(int(i), int(i), *d2[i])
    f.updateParametersInContext(ctx)
    ctx.getState(getEnergy=True, groups={2})
    ref = O.atm_eval(c.spec, c.pos, d2, c.params)
    assert abs(f.getPerturbationEnergy(ctx) - ref["usc"]) <= U_TOL
    # no displacement at all: u = 0 exactly and the ATM force is the state-1 force
    for i in lig:
        f.setParticleParameters(int(i), int(i), 0.0, 0.0, 0.0)
    f.updateParametersInContext(ctx)
    s = ctx.getState(getEnergy=True, getForces=True, groups={2})
    assert f.getPerturbationEnergy(ctx) == 0.0
    E1, F1, _ = O.nonbonded(c.spec, c.pos)
    assert force_rel(s.getForces(), F1) <= F_TOL


def test_batch_results_array_matches_dicts_and_pinned_buffers():
    import torch

    cases = [S.abfe_pme_small(2000, 10, 33), S.abfe_pme_small(2000, 10, 34)]
    b = atm.ReplicaBatch([atm.system_from_case(c)[0] for c in cases], 0)
    pos = np.concatenate([c.pos for c in cases])
    E, F, res = b.evaluate(pos)
    # page-locked caller buffers are copied from and to directly
    pos_pin = torch.from_numpy(pos).pin_memory().numpy()
    F_pin = torch.empty(pos.shape, dtype=torch.float64).pin_memory().numpy()
    E2, F2, arr = b.evaluate(pos_pin, out=F_pin, as_array=True)
    assert F2 is F_pin
    np.testing.assert_array_equal(F2, F)
    np.testing.assert_array_equal(E2, E)
    for k in range(len(cases)):
        assert [res[k][key] for key in atm.RES_KEYS] == arr[k].tolist()
