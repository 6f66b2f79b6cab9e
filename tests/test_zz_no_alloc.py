"""The allocation-free reaction-field entry point against the FP64 oracle.

atm_rf_nonbonded_noalloc serves callers that cannot call cudaMalloc: all of
their device memory comes from their own pool or arena, or allocation is
forbidden while they run.  It must give the NonbondedForce energy and forces of
the FP64 oracle (force RMS relative error <= 1e-4, energy within 2e-6 of the
summed magnitudes of the energy terms) on two calls in a row: its static
scratch is shared between calls and cleared by each, so the second call must
repeat the first bit for bit.  A Context asked for the NonbondedForce's group
(the library's regular path) is checked as well.  The cases include a particle
count that is not a multiple of 32 and particles whose exclusion lists are
empty.  This file sorts last so that a run stopping at the first failure has
run every other test before it.
"""
import copy
import ctypes as C

import numpy as np
import pytest

import atmmetaforce as atm
import oracle as O
from atmmetaforce import _lib
from atmmetaforce import synthetic as S

pytestmark = pytest.mark.gpu

F_TOL = 1e-4


def _torch_cuda():
    try:
        import torch

        return torch if torch.cuda.is_available() else None
    except Exception:
        return None


def _excl_csr(spec):
    n = spec.n
    pairs = [[] for _ in range(n)]
    for i, j in zip(spec.exc_i, spec.exc_j):
        pairs[int(i)].append(int(j))
        pairs[int(j)].append(int(i))
    start = np.zeros(n + 1, dtype=np.int32)
    start[1:] = np.cumsum([len(p) for p in pairs])
    flat = np.array([j for p in pairs for j in p] or [0], dtype=np.int32)
    return start, flat


def _without_exclusions_of(case, atoms):
    """The same system with every exclusion that touches ``atoms`` removed (their
    pairs become ordinary pairs; their exclusion lists are empty)."""
    c = copy.deepcopy(case)
    sp = c.spec
    keep = ~(np.isin(sp.exc_i, atoms) | np.isin(sp.exc_j, atoms))
    for k in ("exc_i", "exc_j", "exc_qq", "exc_sig", "exc_eps"):
        setattr(sp, k, getattr(sp, k)[keep])
    return c


def _noalloc(torch, L, case, calls=2):
    spec = case.spec
    dev = torch.device("cuda", 0)
    torch.cuda.set_device(dev)
    d = lambda a, t=torch.float64: torch.as_tensor(np.ascontiguousarray(a), dtype=t, device=dev)
    pos, q, sg, ep = d(case.pos), d(spec.charge), d(spec.sigma), d(spec.epsilon)
    start, flat = _excl_csr(spec)
    ds, dl = d(start, torch.int32), d(flat, torch.int32)
    box = np.ascontiguousarray(spec.box, dtype=np.float64)
    stream = torch.cuda.current_stream(dev).cuda_stream
    out = []
    for call in range(calls):
        energy = torch.full((1,), float("nan"), dtype=torch.float64, device=dev)
        forces = torch.full((case.n, 3), float("nan"), dtype=torch.float64, device=dev)
        rc = L.atm_rf_nonbonded_noalloc(case.n, pos.data_ptr(), q.data_ptr(), sg.data_ptr(), ep.data_ptr(),
                                        ds.data_ptr(), dl.data_ptr(), box.ctypes.data_as(C.POINTER(C.c_double)),
                                        float(spec.cutoff), float(spec.eps_rf), energy.data_ptr(),
                                        forces.data_ptr(), C.c_void_p(stream))
        assert rc == 0, L.atm_last_error().decode()
        torch.cuda.synchronize()
        out.append((float(energy.item()), forces.cpu().numpy()))
    return out


def _check_against_oracle(case, results):
    E_ref, F_ref, T = O.nonbonded(case.spec, case.pos)
    e_tol = 2e-6 * (sum(abs(v) for v in T.values()) + 1.0)
    for call, (E, F) in enumerate(results):
        assert abs(E - E_ref) <= e_tol, (call, E, E_ref, e_tol)
        rel = np.sqrt(((F - F_ref) ** 2).sum() / (F_ref ** 2).sum())
        assert rel <= F_TOL, (call, rel)
    # the shared scratch is cleared by every call: the second call repeats the first exactly
    assert results[0][0] == results[1][0]
    assert np.array_equal(results[0][1], results[1][1])
    return e_tol


def test_noalloc_matches_oracle_and_context_on_two_calls():
    torch = _torch_cuda()
    if torch is None:
        pytest.skip("no CUDA device")
    case = S.water_ligand_box(3000, 3.1, [16], [(1.4, 1.3, 1.5)], S.CUTOFF_PERIODIC, 0.9, seed=77)
    res = _noalloc(torch, _lib.load(), case)
    e_tol = _check_against_oracle(case, res)

    # second check: the library's regular path (a Context asked for the NonbondedForce's group)
    sys_, nb, f = atm.system_from_case(case)
    ctx = atm.Context(sys_, 0)
    ctx.setPositions(case.pos)
    st = ctx.getState(getEnergy=True, getForces=True, groups={1})
    E_ctx, F_ctx = st.getPotentialEnergy(), st.getForces()
    assert abs(res[0][0] - E_ctx) <= e_tol
    assert np.sqrt(((res[0][1] - F_ctx) ** 2).sum() / (F_ctx ** 2).sum()) <= F_TOL


def test_noalloc_ragged_count_and_empty_exclusion_lists():
    torch = _torch_cuda()
    if torch is None:
        pytest.skip("no CUDA device")
    # 2,993 particles (not a multiple of 32); the last ten waters keep no exclusions
    case = S.water_ligand_box(2993, 3.1, [14], [(1.4, 1.3, 1.5)], S.CUTOFF_PERIODIC, 0.9, seed=78)
    assert case.n % 32 != 0
    n_water = (case.n - 14) // 3
    freed = np.arange(3 * (n_water - 10), 3 * n_water)
    case = _without_exclusions_of(case, freed)
    start, _ = _excl_csr(case.spec)
    assert np.all(start[freed + 1] == start[freed])  # empty lists
    _check_against_oracle(case, _noalloc(torch, _lib.load(), case))


def test_noalloc_rejects_sizes_beyond_its_maximum():
    torch = _torch_cuda()
    if torch is None:
        pytest.skip("no CUDA device")
    L = _lib.load()
    box = np.array([5.0, 5.0, 5.0])
    dummy = torch.zeros(8, dtype=torch.float64, device="cuda")
    idx = torch.zeros(8, dtype=torch.int32, device="cuda")
    rc = L.atm_rf_nonbonded_noalloc(16385, dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(), dummy.data_ptr(),
                                    idx.data_ptr(), idx.data_ptr(), box.ctypes.data_as(C.POINTER(C.c_double)), 0.9,
                                    78.5, dummy.data_ptr(), dummy.data_ptr(), None)
    assert rc == 1
    assert "exceed the maximum" in L.atm_last_error().decode()
