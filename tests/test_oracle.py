"""Known-answer tests of the FP64 oracle (the checker itself is checked here).

Anchors: SoftCoreF and the merge of ReferenceATMMetaForceKernels.cpp:26-113,
closed-form pair energies, an exact Ewald sum for PME, numpy's FFT, and
finite differences of the energy for the forces.
"""
import math

import numpy as np
import pytest

import oracle as O
from atmmetaforce import synthetic as S

K = O.ONE_4PI_EPS0


def two_atom_spec(method, q=(0.5, -0.4), sig=(0.3, 0.34), eps=(0.5, 0.8), box=3.0, cutoff=0.9):
    alpha, grid = (0.0, (0, 0, 0))
    if method == O.PME:
        alpha, grid = S.pme_parameters(cutoff, 5e-4, [box] * 3)
    return S.NonbondedSpec(charge=np.array(q), sigma=np.array(sig), epsilon=np.array(eps),
                           exc_i=np.zeros(0, np.int32), exc_j=np.zeros(0, np.int32), exc_qq=np.zeros(0),
                           exc_sig=np.zeros(0), exc_eps=np.zeros(0), method=method, cutoff=cutoff,
                           box=np.array([box] * 3), alpha=alpha, grid=tuple(grid))


def test_softcore_below_ub_is_identity():
    usc, fp = O.softcore(50.0, 200.0, 0.0625, 100.0)
    assert usc == 50.0 and fp == 1.0


def test_softcore_closed_form_and_derivative():
    umax, a, ub = 200.0, 0.0625, 100.0
    for u in (100.5, 150.0, 400.0, 1e6):
        usc, fp = O.softcore(u, umax, a, ub)
        g = (u - ub) / (a * (umax - ub))
        z = 1 + 2 * g * (g + 1)
        zp = z ** a
        assert usc == pytest.approx((umax - ub) * (zp - 1) / (zp + 1) + ub, rel=1e-14)
        h = 1e-6 * max(1.0, u)
        fd = (O.softcore(u + h, umax, a, ub)[0] - O.softcore(u - h, umax, a, ub)[0]) / (2 * h)
        assert fp == pytest.approx(fd, rel=1e-5)
        assert ub < usc < umax
    # continuity at ub
    assert O.softcore(ub + 1e-9, umax, a, ub)[0] == pytest.approx(ub, abs=1e-8)


@pytest.mark.parametrize("direction", [1.0, -1.0])
def test_merge_matches_reference_formulae(direction):
    p = S.default_params(0.2, 0.7, 0.1, 30.0, 2.0, 200.0, 100.0, 0.0625, direction)
    E1, E2 = -1000.0, -960.0
    F1 = np.random.default_rng(0).normal(size=(5, 3))
    F2 = np.random.default_rng(1).normal(size=(5, 3))
    r = O.atm_merge(E1, E2, p, F1, F2)
    u = E2 - E1 if direction > 0 else E1 - E2
    e0 = E1 if direction > 0 else E2
    ee = 1 + math.exp(-0.1 * (u - 30.0))
    W = (0.7 - 0.2) / 0.1 * math.log(ee) + 0.7 * u + 2.0
    sp = (0.7 - 0.2) / ee + 0.2
    assert r["energy"] == pytest.approx(e0 + W, rel=1e-14)
    assert r["sp"] == pytest.approx(sp, rel=1e-14)
    want = sp * F2 + (1 - sp) * F1 if direction > 0 else sp * F1 + (1 - sp) * F2
    np.testing.assert_allclose(r["forces"], want, rtol=1e-14)
    # sp is dW/du
    h = 1e-5
    Wp = O.atm_merge(E1, E2 + h * direction, p)["W"]
    Wm = O.atm_merge(E1, E2 - h * direction, p)["W"]
    assert (Wp - Wm) / (2 * h) == pytest.approx(sp, rel=1e-7)


def test_merge_alpha_zero_quirk():
    """alpha = 0 drops the log term from W but bfp keeps (l2-l1)/2 + l1
    (ReferenceATMMetaForceKernels.cpp:89-95): dW/du != sp in that corner."""
    p = S.default_params(0.2, 0.6, 0.0, 0.0, 0.0)
    r = O.atm_merge(0.0, 10.0, p)
    assert r["W"] == pytest.approx(0.6 * 10.0)
    assert r["sp"] == pytest.approx((0.6 - 0.2) / 2 + 0.2)


def test_softplus_param_grad_fd():
    p = S.default_params(0.1, 0.45, 0.15, 80.0, 3.0)
    usc = 95.0
    g = O.softplus_param_grad(usc, p)
    for k in range(5):
        h = 1e-6
        pp, pm = p.copy(), p.copy()
        pp[k] += h
        pm[k] -= h
        fd = (O.atm_merge(0, usc, pp)["W"] - O.atm_merge(0, usc, pm)["W"]) / (2 * h)
        assert g[k] == pytest.approx(fd, rel=1e-6, abs=1e-9)


@pytest.mark.parametrize("method", [O.NOCUTOFF, O.CUTOFF_PERIODIC, O.PME])
def test_two_atom_direct_known_answer(method):
    s = two_atom_spec(method)
    r = 0.42
    pos = np.array([[1.0, 1.0, 1.0], [1.0 + r, 1.0, 1.0]])
    E, F, T = O.nonbonded(s, pos)
    sig, eps = 0.32, math.sqrt(0.5 * 0.8)
    qq = 0.5 * -0.4
    lj = 4 * eps * ((sig / r) ** 12 - (sig / r) ** 6)
    if method == O.NOCUTOFF:
        coul = K * qq / r
    elif method == O.CUTOFF_PERIODIC:
        krf = (78.5 - 1) / ((2 * 78.5 + 1) * 0.9 ** 3)
        crf = 3 * 78.5 / ((2 * 78.5 + 1) * 0.9)
        coul = K * qq * (1 / r + krf * r * r - crf)
    else:
        coul = K * qq * math.erfc(s.alpha * r) / r
    assert T["direct"] == pytest.approx(lj + coul, rel=1e-12)
    # Newton's third law and finite difference of the direct term
    h = 1e-6
    p2 = pos.copy(); p2[1, 0] += h
    p3 = pos.copy(); p3[1, 0] -= h
    fd = -(O.nonbonded(s, p2)[2]["direct"] - O.nonbonded(s, p3)[2]["direct"]) / (2 * h)
    if method != O.PME:
        assert F[1, 0] == pytest.approx(fd, rel=1e-6)
        np.testing.assert_allclose(F[0], -F[1], atol=1e-9)


def test_cutoff_excludes_pairs_beyond_rc():
    s = two_atom_spec(O.CUTOFF_PERIODIC)
    pos = np.array([[0.2, 0.2, 0.2], [1.15, 0.2, 0.2]])
    E, F, T = O.nonbonded(s, pos)
    assert T["direct"] == 0.0
    # minimum image: 0.2 and 2.9 are 0.3 apart in a 3.0 box
    pos = np.array([[0.2, 0.2, 0.2], [2.9, 0.2, 0.2]])
    assert O.nonbonded(s, pos)[2]["direct"] != 0.0


def test_fft_matches_numpy():
    rng = np.random.default_rng(5)
    for dims in ((8, 6, 10), (7, 9, 5), (38, 42, 39)):
        a = rng.normal(size=dims) + 1j * rng.normal(size=dims)
        np.testing.assert_allclose(O.fft3d(a, -1), np.fft.fftn(a), rtol=1e-10, atol=1e-9)
        np.testing.assert_allclose(O.fft3d(a, +1), np.fft.ifftn(a) * a.size, rtol=1e-10, atol=1e-9)


def test_pme_grid_rule():
    a, g = S.pme_parameters(0.9, 5e-4, [6.2] * 3)
    assert g == [56, 56, 56] and a == pytest.approx(math.sqrt(-math.log(1e-3)) / 0.9)
    a2, g2 = O.pme_parameters(0.9, 5e-4, [6.2] * 3)
    assert g2 == g and a2 == pytest.approx(a)
    _, g3 = S.pme_parameters(1.0, 5e-4, [4.6742747, 5.1635997, 4.8361653], legal=True)
    assert g3 == [40, 42, 40]


def test_pme_converges_to_exact_ewald():
    c = S.abfe_pme_small(900, 12, 3)
    Ee, Fe = O.ewald_recip_exact(c.spec, c.pos, 14)
    E, F, T = O.nonbonded(c.spec, c.pos)
    # at the tolerance grid the SPME error is a few 1e-4 relative
    assert abs(T["recip"] - Ee) < 5e-4 * abs(Ee) + 0.5
    import copy
    fine = copy.copy(c.spec)
    fine.grid = (64, 64, 64)
    _, _, Tf = O.nonbonded(fine, c.pos)
    assert abs(Tf["recip"] - Ee) < 2e-6 * abs(Ee) + 1e-3


@pytest.mark.parametrize("builder", ["rf", "pme"])
def test_forces_are_minus_energy_gradient(builder):
    c = S.abfe_rf_2394(0) if builder == "rf" else S.abfe_pme_small(900, 12, 3)
    E, F, _ = O.nonbonded(c.spec, c.pos)
    rng = np.random.default_rng(9)
    h = 1e-5
    for i in list(rng.choice(c.n, 4, replace=False)) + [c.n - 1]:
        for a in range(3):
            p = c.pos.copy(); p[i, a] += h
            Ep = O.nonbonded(c.spec, p, pos_cut=c.pos, forces=False)[0]
            p[i, a] -= 2 * h
            Em = O.nonbonded(c.spec, p, pos_cut=c.pos, forces=False)[0]
            assert -(Ep - Em) / (2 * h) == pytest.approx(F[i, a], rel=2e-5, abs=2e-3)


def test_param_derivs_fd():
    c = S.abfe_pme_small(900, 12, 4)
    dq, ds, de = O.param_derivs(c.spec, c.pos)
    import copy
    for i in (c.ligands[0][0], c.ligands[0][5], 3):
        for arr, d in (("charge", dq), ("sigma", ds), ("epsilon", de)):
            h = 1e-6
            sp, sm = copy.copy(c.spec), copy.copy(c.spec)
            a = getattr(c.spec, arr).copy(); a[i] += h; setattr(sp, arr, a)
            b = getattr(c.spec, arr).copy(); b[i] -= h; setattr(sm, arr, b)
            fd = (O.nonbonded(sp, c.pos, forces=False)[0] - O.nonbonded(sm, c.pos, forces=False)[0]) / (2 * h)
            assert d[i] == pytest.approx(fd, rel=1e-5, abs=1e-4), (arr, i)


def test_atm_eval_is_two_states_plus_merge():
    c = S.abfe_rf_2394(0)
    r = O.atm_eval(c.spec, c.pos, c.displ, c.params, want_states=True)
    E1, F1, _ = O.nonbonded(c.spec, c.pos)
    E2, F2, _ = O.nonbonded(c.spec, c.pos + c.displ)
    assert r["E1"] == pytest.approx(E1, rel=1e-14) and r["E2"] == pytest.approx(E2, rel=1e-14)
    m = O.atm_merge(E1, E2, c.params, F1, F2)
    np.testing.assert_allclose(r["forces"], m["forces"], rtol=1e-13, atol=1e-10)
    assert r["usc"] == pytest.approx(m["usc"])


def test_threads_do_not_change_results():
    c = S.abfe_pme_small(900, 12, 6)
    O.set_threads(1)
    E1, F1, _ = O.nonbonded(c.spec, c.pos)
    O.set_threads(4)
    E4, F4, _ = O.nonbonded(c.spec, c.pos)
    O.set_threads(1)
    assert E4 == pytest.approx(E1, rel=1e-12)
    np.testing.assert_allclose(F4, F1, rtol=1e-9, atol=1e-9)


# ---------------------------------------------------------------------------
# Triclinic boxes (OpenMM's reduced form a = (ax,0,0), b = (bx,by,0), c = (cx,cy,cz))
# ---------------------------------------------------------------------------

TILTS = [(0.9, -0.7, 0.8), (1.4, 1.3, -1.2)]


@pytest.mark.parametrize("tilt", TILTS)
def test_triclinic_pme_matches_exact_ewald(tilt):
    import copy

    c = S.triclinic_water_ligand_box(3000, (3.2, 3.0, 2.9), tilt, [14], [(1.3, 1.2, 1.1)], S.PME, 0.9, seed=5)
    fine = copy.copy(c.spec)
    fine.grid = tuple(2 * g for g in c.spec.grid)
    E_pme = O.nonbonded(fine, c.pos, forces=False)[2]["recip"]
    E_exact, _ = O.ewald_recip_exact(c.spec, c.pos, 16)
    assert abs(E_pme - E_exact) < 0.05, (E_pme, E_exact)


@pytest.mark.parametrize("method", [S.PME, S.CUTOFF_PERIODIC])
def test_triclinic_forces_are_energy_gradients(method):
    c = S.triclinic_water_ligand_box(600, (2.1, 2.0, 1.95), (0.7, -0.6, 0.5), [8], [(0.9, 0.8, 0.7)], method, 0.9,
                                     seed=6)
    E, F, _ = O.nonbonded(c.spec, c.pos)
    h = 1e-5
    rng = np.random.default_rng(0)
    for i in rng.choice(c.n, 6, replace=False):
        for d in range(3):
            p1, p2 = c.pos.copy(), c.pos.copy()
            p1[i, d] += h
            p2[i, d] -= h
            # the pair set stays that of the unperturbed geometry
            fd = -(O.nonbonded(c.spec, p1, pos_cut=c.pos, forces=False)[0] -
                   O.nonbonded(c.spec, p2, pos_cut=c.pos, forces=False)[0]) / (2 * h)
            assert abs(F[i, d] - fd) <= 1e-5 * max(1.0, abs(fd)), (i, d, F[i, d], fd)


def test_triclinic_direct_space_matches_image_search():
    """Reaction field over the pairs within the cutoff, the pair vector being the
    shortest over the 125 images next to the reduced-form minimum image."""
    c = S.triclinic_water_ligand_box(900, (2.3, 2.2, 2.1), (0.9, -0.8, 0.7), [8], [(1.0, 0.9, 0.8)],
                                     S.CUTOFF_PERIODIC, 0.9, seed=7)
    sp = c.spec
    _, _, T = O.nonbonded(sp, c.pos, forces=False)
    B = S.box_vectors(sp.box, sp.tilt)
    shifts = np.array([(i, j, k) for i in range(-2, 3) for j in range(-2, 3) for k in range(-2, 3)]) @ B
    excl = set(zip(sp.exc_i.tolist(), sp.exc_j.tolist())) | set(zip(sp.exc_j.tolist(), sp.exc_i.tolist()))
    rc, er = sp.cutoff, sp.eps_rf
    krf = (er - 1) / ((2 * er + 1) * rc ** 3)
    crf = 3 * er / ((2 * er + 1) * rc)
    E = 0.0
    for i in range(c.n):
        d = c.pos[i + 1:] - c.pos[i]
        dd = d[:, None, :] + shifts[None, :, :]
        r2 = (dd * dd).sum(-1).min(axis=1)
        for jj in np.nonzero(r2 < rc * rc)[0]:
            j = i + 1 + jj
            if (i, j) in excl:
                continue
            r = np.sqrt(r2[jj])
            sig = 0.5 * (sp.sigma[i] + sp.sigma[j])
            eps = np.sqrt(sp.epsilon[i] * sp.epsilon[j])
            s6 = (sig / r) ** 6
            E += 4 * eps * (s6 * s6 - s6) + O.ONE_4PI_EPS0 * sp.charge[i] * sp.charge[j] * (1 / r + krf * r * r - crf)
    assert abs(T["direct"] - E) <= 1e-8 * max(1.0, abs(E)), (T["direct"], E)
