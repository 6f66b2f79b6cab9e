"""Adjoint of the ATM softplus bias energy W against the FP64 oracle.

Checks dW/d(positions), dW/d(displacement), dW/d(ligand q, sigma, eps) and the
five softplus parameters against (a) the oracle's analytic gradient and
(b) central finite differences of W computed in FP64 (h = 1e-4; the pair set
is frozen at the unperturbed geometry so that the plain cutoff does not make
W jump).  Tolerance: 1e-3 relative, with no absolute floor; the finite
differences are taken on the components where the analytic gradient is largest
(softplus parameters whose derivative lies below the finite differences' noise
floor, 1e-6 max(1, |W|), are skipped).
Cases: two 3,000-atom boxes (directions +1 and -1), and the batch of eight
12,000-atom PME boxes with 30-atom ligands displaced by (2,2,2) nm.
"""
import copy
import os

import numpy as np
import pytest

import atmmetaforce as atm
import oracle as O
from atmmetaforce import synthetic as S

pytestmark = pytest.mark.gpu

REL = 1e-3
H = 1e-4


def _has_gpu():
    try:
        import torch

        return torch.cuda.is_available()
    except Exception:
        return False


if not _has_gpu():
    pytest.skip("no CUDA device", allow_module_level=True)


@pytest.fixture(scope="module")
def setup():
    O.set_threads(min(16, os.cpu_count() or 1))
    rng = np.random.default_rng(5)
    cases = []
    for k in range(2):
        c = S.water_ligand_box(3000, 3.1, [14], [(1.3, 1.4, 1.5)], S.PME, 0.9, seed=70 + k)
        l1, l2 = rng.uniform(0, 0.5, 2)
        c.params = S.default_params(l1, l2, rng.uniform(0.05, 0.2), rng.uniform(-60, 60), 1.0, 200.0, 100.0,
                                    0.0625, 1.0 if k == 0 else -1.0)
        cases.append(c)
    systems = [atm.system_from_case(c)[0] for c in cases]
    b = atm.ReplicaBatch(systems, 0, {"DifferencePath": 1, "Adjoint": 1})
    E, F, res = b.evaluate(np.concatenate([c.pos for c in cases]))
    grads = b.backward()
    yield cases, b, res, grads
    O.set_threads(1)


def W_of(spec, pos, displ, params, pos_cut, cut_displ):
    E1 = O.nonbonded(spec, pos, pos_cut=pos_cut, forces=False)[0]
    E2 = O.nonbonded(spec, pos + displ, pos_cut=pos_cut + cut_displ, forces=False)[0]
    return O.atm_merge(E1, E2, params)["W"]


def oracle_grads(c):
    r = O.atm_eval(c.spec, c.pos, c.displ, c.params, want_states=True)
    m = O.atm_merge(r["E1"], r["E2"], c.params)
    s = 1.0 if c.params[8] > 0 else -1.0
    dWdu = (m["bfp"] if c.params[2] > 0 else c.params[1]) * m["fp"]
    dq1, ds1, de1 = O.param_derivs(c.spec, c.pos)
    dq2, ds2, de2 = O.param_derivs(c.spec, c.pos + c.displ)
    return {
        "positions": -s * dWdu * (r["F2"] - r["F1"]),
        "displacements": -s * dWdu * r["F2"],
        "charge": s * dWdu * (dq2 - dq1),
        "sigma": s * dWdu * (ds2 - ds1),
        "epsilon": s * dWdu * (de2 - de1),
        "params": O.softplus_param_grad(m["usc"], c.params),
        "W": m["W"],
    }


def rel_err(a, b):
    return float(np.linalg.norm(np.asarray(a) - np.asarray(b)) / max(np.linalg.norm(b), 1e-12))


def test_adjoint_matches_analytic_oracle_gradient(setup):
    cases, b, res, grads = setup
    for k, c in enumerate(cases):
        ref = oracle_grads(c)
        a, z = b.offsets[k], b.offsets[k + 1]
        assert abs(res[k]["W"] - ref["W"]) <= 0.01 * max(1.0, abs(c.params[1]))
        lig = c.ligands[0]
        for key in ("positions", "displacements"):
            assert rel_err(grads[key][a:z], ref[key]) <= REL, key
        for key in ("charge", "sigma", "epsilon"):
            assert rel_err(grads[key][a:z][lig], ref[key][lig]) <= REL, key
        assert rel_err(grads["params"][k], ref["params"]) <= REL


def _top(v, k):
    """Indices of the k entries of v largest in magnitude."""
    return np.argsort(-np.abs(np.asarray(v).ravel()), kind="stable")[:k]


def fd_check(c, grads, k, a, ref, n_pos=6, n_displ=4, n_param_atoms=2):
    """Central differences of W (FP64 oracle, h = 1e-4, pair set frozen at the
    unperturbed geometry) against the GPU adjoint of replica k (atoms from offset
    a), on the components where the analytic gradient is largest: a relative
    bound is only meaningful away from zero.  Returns the largest relative error."""
    worst = 0.0
    lig = c.ligands[0]

    def check(got, fd, what):
        nonlocal worst
        err = abs(got - fd) / abs(fd)
        worst = max(worst, err)
        assert err <= REL, (what, got, fd)

    for flat in _top(ref["positions"], n_pos):
        i, d = divmod(int(flat), 3)
        p1, p2 = c.pos.copy(), c.pos.copy()
        p1[i, d] += H
        p2[i, d] -= H
        fd = (W_of(c.spec, p1, c.displ, c.params, c.pos, c.displ) -
              W_of(c.spec, p2, c.displ, c.params, c.pos, c.displ)) / (2 * H)
        check(grads["positions"][a + i, d], fd, ("position", i, d))
    for flat in _top(ref["displacements"][lig], n_displ):
        m, d = divmod(int(flat), 3)
        i = int(lig[m])
        d1, d2 = c.displ.copy(), c.displ.copy()
        d1[i, d] += H
        d2[i, d] -= H
        fd = (W_of(c.spec, c.pos, d1, c.params, c.pos, c.displ) -
              W_of(c.spec, c.pos, d2, c.params, c.pos, c.displ)) / (2 * H)
        check(grads["displacements"][a + i, d], fd, ("displacement", i, d))
    for key in ("charge", "sigma", "epsilon"):
        for m in _top(ref[key][lig], n_param_atoms):
            i = int(lig[m])
            s1, s2 = copy.copy(c.spec), copy.copy(c.spec)
            v1 = getattr(c.spec, key).copy()
            v2 = v1.copy()
            v1[i] += H
            v2[i] -= H
            setattr(s1, key, v1)
            setattr(s2, key, v2)
            fd = (W_of(s1, c.pos, c.displ, c.params, c.pos, c.displ) -
                  W_of(s2, c.pos, c.displ, c.params, c.pos, c.displ)) / (2 * H)
            check(grads[key][a + i], fd, (key, i))
    # softplus parameters: the finite difference of W alone has a noise floor of
    # about 1e-14 |W| / h; a component far below it (dW/du0 vanishes when
    # alpha (usc - u0) >> 1) cannot be checked to a relative bound
    floor = 1e-6 * max(1.0, abs(ref["W"]))
    for p in range(5):
        if abs(ref["params"][p]) < floor:
            continue
        q1, q2 = c.params.copy(), c.params.copy()
        q1[p] += H
        q2[p] -= H
        fd = (W_of(c.spec, c.pos, c.displ, q1, c.pos, c.displ) -
              W_of(c.spec, c.pos, c.displ, q2, c.pos, c.displ)) / (2 * H)
        check(grads["params"][k, p], fd, ("param", p))
    return worst


def test_adjoint_matches_finite_differences(setup):
    cases, b, res, grads = setup
    for k in (0, 1):
        fd_check(cases[k], grads, k, b.offsets[k], oracle_grads(cases[k]))


@pytest.fixture(scope="module")
def batch8():
    """8 seeded 12,000-atom PME boxes, 30-atom ligands displaced by (2,2,2) nm,
    softplus parameters lambda U[0,0.5], alpha U[0,0.2], u0 U[50,150]."""
    O.set_threads(min(16, os.cpu_count() or 1))
    cases = S.adjoint_batch_8()
    b = atm.ReplicaBatch([atm.system_from_case(c)[0] for c in cases], 0, {"DifferencePath": 1, "Adjoint": 1})
    E, F, res = b.evaluate(np.concatenate([c.pos for c in cases]))
    grads = b.backward()
    yield cases, b, res, grads
    O.set_threads(1)


def test_adjoint_batch_of_eight_12000_atom_boxes_analytic(batch8):
    cases, b, res, grads = batch8
    worst = 0.0
    for k, c in enumerate(cases):
        ref = oracle_grads(c)
        a, z = b.offsets[k], b.offsets[k + 1]
        assert res[k]["status"] == 0
        lig = c.ligands[0]
        errs = [rel_err(grads["positions"][a:z], ref["positions"]),
                rel_err(grads["displacements"][a:z], ref["displacements"]),
                rel_err(grads["params"][k], ref["params"])]
        errs += [rel_err(grads[key][a:z][lig], ref[key][lig]) for key in ("charge", "sigma", "epsilon")]
        worst = max(worst, max(errs))
        assert max(errs) <= REL, (k, errs)
    print(f"8 x 12,000 adjoint: largest relative error against the analytic oracle gradient {worst:.2e}")


def test_adjoint_batch_of_eight_12000_atom_boxes_finite_differences(batch8):
    cases, b, res, grads = batch8
    worst = 0.0
    for k in (0, 7):
        worst = max(worst, fd_check(cases[k], grads, k, b.offsets[k], oracle_grads(cases[k])))
    print(f"8 x 12,000 adjoint: largest relative error against central differences {worst:.2e}")


def test_torch_autograd_function_wires_the_adjoint(setup):
    import torch

    from atmmetaforce.autograd import atm_softplus_energy, batch_tensors

    cases, b, res, grads = setup
    pos, displ, params, q, s, e = batch_tensors(b and b, cases)
    for t in (pos, displ, params, q, s, e):
        t.requires_grad_(True)
    W = atm_softplus_energy(b, pos, displ, params, q, s, e)
    gw = torch.tensor([1.0, 0.5], dtype=torch.float64, device=W.device)
    (W * gw).sum().backward()
    assert np.allclose(W.detach().cpu().numpy(), [r["W"] for r in res], rtol=1e-12, atol=1e-9)
    for k in range(2):
        a, z = b.offsets[k], b.offsets[k + 1]
        np.testing.assert_allclose(pos.grad[a:z].cpu().numpy(), gw[k].item() * grads["positions"][a:z], rtol=1e-9,
                                   atol=1e-9)
        np.testing.assert_allclose(q.grad[a:z].cpu().numpy(), gw[k].item() * grads["charge"][a:z], rtol=1e-9,
                                   atol=1e-9)
    np.testing.assert_allclose(params.grad.cpu().numpy()[1], 0.5 * grads["params"][1], rtol=1e-9, atol=1e-12)
