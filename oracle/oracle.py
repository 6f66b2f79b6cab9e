"""ctypes front of the FP64 CPU oracle (oracle/atm_oracle.c).

TEST INFRASTRUCTURE ONLY.  Imported by tests/, by ``__graft_entry__.smoke()`` and
by the CPU-baseline leg of ``bench.py``; never by the product package.

The oracle restates the reference's Reference-platform ATM merge
(platforms/reference/src/ReferenceATMMetaForceKernels.cpp:26-157) and the inner
NonbondedForce evaluation the reference delegates to OpenMM
(openmmapi/src/ATMMetaForceImpl.cpp:113,116).

A "spec" is any object with the attributes charge, sigma, epsilon (arrays),
exc_i, exc_j, exc_qq, exc_sig, exc_eps (arrays), method, cutoff, eps_rf, alpha,
grid (3 ints), order, use_disp_corr, box (3 floats: the diagonal of the box
vectors) and optionally tilt (b_x, c_x, c_y of OpenMM's reduced triclinic box
vectors a = (box0, 0, 0), b = (b_x, box1, 0), c = (c_x, c_y, box2)).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(HERE, "_build", "liboracle.so")

NOCUTOFF, CUTOFF_NONPERIODIC, CUTOFF_PERIODIC, PME = 0, 1, 2, 4
ONE_4PI_EPS0 = 138.935456

_dp = C.POINTER(C.c_double)
_ip = C.POINTER(C.c_int)


class _ONB(C.Structure):
    _fields_ = [
        ("n", C.c_int),
        ("charge", _dp), ("sigma", _dp), ("epsilon", _dp),
        ("n_exc", C.c_int),
        ("exc_i", _ip), ("exc_j", _ip),
        ("exc_qq", _dp), ("exc_sig", _dp), ("exc_eps", _dp),
        ("method", C.c_int),
        ("cutoff", C.c_double),
        ("eps_rf", C.c_double),
        ("alpha", C.c_double),
        ("grid", C.c_int * 3),
        ("order", C.c_int),
        ("use_disp_corr", C.c_int),
        ("box", C.c_double * 3),
        ("tilt", C.c_double * 3),
    ]


class _Terms(C.Structure):
    _fields_ = [("direct", C.c_double), ("exceptions", C.c_double), ("recip", C.c_double),
                ("self", C.c_double), ("disp", C.c_double)]


_lib = None


def build(force: bool = False) -> str:
    """Compile the oracle with its Makefile (gcc, OpenMP)."""
    if force or not os.path.exists(LIB_PATH):
        subprocess.run(["make", "-s", "-C", HERE], check=True)
    return LIB_PATH


def lib():
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            build()
        L = C.CDLL(LIB_PATH)
        L.onb_energy_forces.argtypes = [C.POINTER(_ONB), _dp, _dp, _dp, _dp, C.POINTER(_Terms)]
        L.onb_param_derivs.argtypes = [C.POINTER(_ONB), _dp, _dp, _dp, _dp, _dp]
        L.onb_ewald_recip_exact.argtypes = [C.POINTER(_ONB), _dp, C.c_int, _dp, _dp]
        L.o_softcore.argtypes = [C.c_double] * 4 + [_dp]
        L.o_softcore.restype = C.c_double
        L.o_atm_merge.argtypes = [C.c_double, C.c_double, _dp, C.c_int, _dp, _dp, _dp, _dp]
        L.o_softplus_param_grad.argtypes = [C.c_double, _dp, _dp]
        L.o_atm_eval.argtypes = [C.POINTER(_ONB), _dp, _dp, _dp, _dp, _dp, _dp, _dp, _dp]
        L.o_pme_parameters.argtypes = [C.c_double, C.c_double, _dp, C.c_int, _dp, _ip]
        L.o_fft3d.argtypes = [_dp, _ip, C.c_int]
        L.o_set_threads.argtypes = [C.c_int]
        _lib = L
    return _lib


def set_threads(n: int) -> int:
    return lib().o_set_threads(int(n))


def _d(a):
    return np.ascontiguousarray(a, dtype=np.float64)


def _ptr(a, t=_dp):
    return a.ctypes.data_as(t) if a is not None else None


class _Pinned:
    """Keeps the numpy arrays referenced by an _ONB struct alive."""

    def __init__(self, spec):
        self.q = _d(spec.charge)
        self.s = _d(spec.sigma)
        self.e = _d(spec.epsilon)
        self.ei = np.ascontiguousarray(spec.exc_i, dtype=np.int32)
        self.ej = np.ascontiguousarray(spec.exc_j, dtype=np.int32)
        self.eqq = _d(spec.exc_qq)
        self.esig = _d(spec.exc_sig)
        self.eeps = _d(spec.exc_eps)
        o = _ONB()
        o.n = len(self.q)
        o.charge, o.sigma, o.epsilon = _ptr(self.q), _ptr(self.s), _ptr(self.e)
        o.n_exc = len(self.ei)
        o.exc_i, o.exc_j = _ptr(self.ei, _ip), _ptr(self.ej, _ip)
        o.exc_qq, o.exc_sig, o.exc_eps = _ptr(self.eqq), _ptr(self.esig), _ptr(self.eeps)
        o.method = int(spec.method)
        o.cutoff = float(spec.cutoff)
        o.eps_rf = float(spec.eps_rf)
        o.alpha = float(spec.alpha)
        tilt = getattr(spec, "tilt", None)
        for a in range(3):
            o.grid[a] = int(spec.grid[a])
            o.box[a] = float(spec.box[a])
            o.tilt[a] = float(tilt[a]) if tilt is not None else 0.0
        o.order = int(spec.order)
        o.use_disp_corr = int(spec.use_disp_corr)
        self.struct = o


def nonbonded(spec, pos, pos_cut=None, forces=True):
    """Energy (kJ/mol), forces (kJ/mol/nm, n x 3) and the energy terms."""
    P = _Pinned(spec)
    pos = _d(pos).reshape(-1, 3)
    pc = _d(pos_cut).reshape(-1, 3) if pos_cut is not None else None
    e = C.c_double()
    F = np.zeros_like(pos) if forces else None
    t = _Terms()
    rc = lib().onb_energy_forces(C.byref(P.struct), _ptr(pos), _ptr(pc), C.byref(e), _ptr(F), C.byref(t))
    if rc:
        raise RuntimeError(f"oracle nonbonded failed ({rc})")
    terms = dict(direct=t.direct, exceptions=t.exceptions, recip=t.recip, self=t.self, disp=t.disp)
    return e.value, F, terms


def param_derivs(spec, pos, pos_cut=None):
    """dU/dq, dU/dsigma, dU/depsilon per particle."""
    P = _Pinned(spec)
    pos = _d(pos).reshape(-1, 3)
    pc = _d(pos_cut).reshape(-1, 3) if pos_cut is not None else None
    n = len(P.q)
    dq, ds, de = np.zeros(n), np.zeros(n), np.zeros(n)
    rc = lib().onb_param_derivs(C.byref(P.struct), _ptr(pos), _ptr(pc), _ptr(dq), _ptr(ds), _ptr(de))
    if rc:
        raise RuntimeError(f"oracle param_derivs failed ({rc})")
    return dq, ds, de


def ewald_recip_exact(spec, pos, kmax):
    P = _Pinned(spec)
    pos = _d(pos).reshape(-1, 3)
    e = C.c_double()
    F = np.zeros_like(pos)
    lib().onb_ewald_recip_exact(C.byref(P.struct), _ptr(pos), int(kmax), C.byref(e), _ptr(F))
    return e.value, F


def softcore(u, umax, acore, ubcore):
    fp = C.c_double()
    usc = lib().o_softcore(float(u), float(umax), float(acore), float(ubcore), C.byref(fp))
    return usc, fp.value


MERGE_KEYS = ("energy", "usc", "sp", "W", "u", "e0", "bfp", "fp")


def atm_merge(E1, E2, params, F1=None, F2=None):
    p = _d(params)
    out = np.zeros(8)
    n = 0 if F1 is None else len(np.asarray(F1).reshape(-1, 3))
    f1 = _d(F1).reshape(-1) if F1 is not None else None
    f2 = _d(F2).reshape(-1) if F2 is not None else None
    fo = np.zeros(3 * n) if n else None
    lib().o_atm_merge(float(E1), float(E2), _ptr(p), n, _ptr(f1), _ptr(f2), _ptr(fo), _ptr(out))
    res = dict(zip(MERGE_KEYS, out.tolist()))
    if n:
        res["forces"] = fo.reshape(-1, 3)
    return res


def softplus_param_grad(usc, params):
    out = np.zeros(5)
    lib().o_softplus_param_grad(float(usc), _ptr(_d(params)), _ptr(out))
    return out


def atm_eval(spec, pos, displ, params, pos_cut=None, want_states=False):
    """Full ATM evaluation: dict with energy, usc, sp, W, u, e0, bfp, fp, forces
    (and E1, E2, F1, F2 when want_states)."""
    P = _Pinned(spec)
    pos = _d(pos).reshape(-1, 3)
    d = _d(displ).reshape(-1, 3)
    pc = _d(pos_cut).reshape(-1, 3) if pos_cut is not None else None
    n = len(pos)
    F = np.zeros_like(pos)
    out = np.zeros(8)
    E12 = np.zeros(2)
    F12 = np.zeros(6 * n) if want_states else None
    rc = lib().o_atm_eval(C.byref(P.struct), _ptr(pos), _ptr(d), _ptr(_d(params)), _ptr(pc), _ptr(F),
                          _ptr(out), _ptr(E12), _ptr(F12))
    if rc:
        raise RuntimeError(f"oracle atm_eval failed ({rc})")
    res = dict(zip(MERGE_KEYS, out.tolist()))
    res["forces"] = F
    res["E1"], res["E2"] = E12.tolist()
    if want_states:
        res["F1"] = F12[: 3 * n].reshape(-1, 3)
        res["F2"] = F12[3 * n:].reshape(-1, 3)
    return res


def pme_parameters(cutoff, tol, box, legal=False):
    a = C.c_double()
    g = (C.c_int * 3)()
    b = _d(box)
    lib().o_pme_parameters(float(cutoff), float(tol), _ptr(b), int(bool(legal)), C.byref(a), g)
    return a.value, [g[0], g[1], g[2]]


def fft3d(arr, sign=-1):
    """Complex 3D FFT of the oracle (unnormalised); sign -1 forward."""
    a = np.ascontiguousarray(arr, dtype=np.complex128).copy()
    dims = (C.c_int * 3)(*a.shape)
    lib().o_fft3d(a.ctypes.data_as(_dp), dims, int(sign))
    return a
