"""Python API of the GB300 ATM path, mirroring the reference's SWIG module.

``ATMMetaForce`` has the methods of python/atmmetaforceplugin.i:64-124 (same
names, argument order and meaning; lengths in nm, energies in kJ/mol as plain
floats: there is no openmm.unit here).  ``NonbondedForce``, ``System`` and
``Context`` stand in for the OpenMM classes the reference plugs into, limited to
what the ATM path uses.  ``ReplicaBatch`` evaluates many replicas in one CUDA
graph.  Every call goes through the C ABI of include/atm_capi.h.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from . import _lib
from ._lib import ATMError, NUM_RES, RES_KEYS, call

_dp = C.POINTER(C.c_double)


def _ptr(a):
    return a.ctypes.data_as(_dp)


def _vec3(v):
    return np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(3))


class ATMMetaForce:
    """The ATM meta-force (openmmapi/include/ATMMetaForce.h:54-315)."""

    def __init__(self, lambda1, lambda2, alpha, u0, w0, umax, ubcore, acore, direction, variableForceGroups=(),
                 _handle=None):
        if _handle is not None:
            self._h = _handle
        else:
            g = np.ascontiguousarray(list(variableForceGroups), dtype=np.int32)
            h = C.c_void_p()
            call("atm_force_create", float(lambda1), float(lambda2), float(alpha), float(u0), float(w0),
                 float(umax), float(ubcore), float(acore), float(direction),
                 g.ctypes.data_as(C.POINTER(C.c_int)), len(g), C.byref(h))
            self._h = h
        self._owned = True  # by this object until added to a System

    def __del__(self):
        try:
            if getattr(self, "_owned", False) and self._h:
                _lib.load().atm_force_destroy(self._h)
        except Exception:
            pass

    # -- static names (ATMMetaForce.h:151-227) --
    @staticmethod
    def Lambda1():
        return "ATMLambda1"

    @staticmethod
    def Lambda2():
        return "ATMLambda2"

    @staticmethod
    def Alpha():
        return "ATMAlpha"

    @staticmethod
    def U0():
        return "ATMU0"

    @staticmethod
    def W0():
        return "ATMW0"

    @staticmethod
    def Umax():
        return "ATMUmax"

    @staticmethod
    def Ubcore():
        return "ATMUbcore"

    @staticmethod
    def Acore():
        return "ATMAcore"

    @staticmethod
    def Direction():
        return "ATMDirection"

    @staticmethod
    def Version():
        return _lib.load().atm_version().decode()

    # -- particles --
    def getNumParticles(self):
        n = C.c_int()
        call("atm_force_get_num_particles", self._h, C.byref(n))
        return n.value

    def addParticle(self, particle, dx=0.0, dy=0.0, dz=0.0):
        k = C.c_int()
        call("atm_force_add_particle", self._h, int(particle), float(dx), float(dy), float(dz), C.byref(k))
        return k.value

    def getParticleParameters(self, index):
        p = C.c_int()
        dx, dy, dz = C.c_double(), C.c_double(), C.c_double()
        call("atm_force_get_particle_parameters", self._h, int(index), C.byref(p), C.byref(dx), C.byref(dy),
             C.byref(dz))
        return [p.value, dx.value, dy.value, dz.value]

    def setParticleParameters(self, index, particle, dx, dy, dz):
        call("atm_force_set_particle_parameters", self._h, int(index), int(particle), float(dx), float(dy), float(dz))

    def updateParametersInContext(self, context):
        call("atm_force_update_parameters_in_context", self._h, context._h)

    def getPerturbationEnergy(self, context):
        v = C.c_double()
        call("atm_force_get_perturbation_energy", self._h, context._h, C.byref(v))
        return v.value

    def usesPeriodicBoundaryConditions(self):
        u = C.c_int()
        call("atm_force_uses_periodic_boundary_conditions", self._h, C.byref(u))
        return bool(u.value)

    # -- defaults --
    def _default(self, k):
        v = C.c_double()
        call("atm_force_get_default", self._h, k, C.byref(v))
        return v.value

    def getDefaultLambda1(self):
        return self._default(0)

    def getDefaultLambda2(self):
        return self._default(1)

    def getDefaultAlpha(self):
        return self._default(2)

    def getDefaultU0(self):
        return self._default(3)

    def getDefaultW0(self):
        return self._default(4)

    def getDefaultUmax(self):
        return self._default(5)

    def getDefaultUbcore(self):
        return self._default(6)

    def getDefaultAcore(self):
        return self._default(7)

    def getDefaultDirection(self):
        return self._default(8)

    def getVariableForceGroups(self):
        n = C.c_int()
        call("atm_force_get_variable_force_groups", self._h, None, 0, C.byref(n))
        buf = (C.c_int * max(1, n.value))()
        call("atm_force_get_variable_force_groups", self._h, buf, n.value, C.byref(n))
        return [buf[k] for k in range(n.value)]

    # -- Force base class --
    def setForceGroup(self, g):
        call("atm_force_set_force_group", self._h, int(g))

    def getForceGroup(self):
        g = C.c_int()
        call("atm_force_get_force_group", self._h, C.byref(g))
        return g.value

    def setName(self, name):
        call("atm_force_set_name", self._h, name.encode())

    def getName(self):
        n = C.c_size_t()
        call("atm_force_get_name", self._h, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value + 1)
        call("atm_force_get_name", self._h, buf, n.value + 1, C.byref(n))
        return buf.value.decode()

    # -- XML (serialization/src/ATMMetaForceProxy.cpp) --
    def serialize(self):
        n = C.c_size_t()
        call("atm_force_serialize", self._h, None, 0, C.byref(n))
        buf = C.create_string_buffer(n.value + 1)
        call("atm_force_serialize", self._h, buf, n.value + 1, C.byref(n))
        return buf.value.decode()

    @staticmethod
    def deserialize(xml):
        h = C.c_void_p()
        call("atm_force_deserialize", xml.encode(), C.byref(h))
        return ATMMetaForce(0, 0, 0, 0, 0, 0, 0, 0, 0, _handle=h)

    @staticmethod
    def isinstance(force):
        return isinstance(force, ATMMetaForce)

    @staticmethod
    def cast(force):
        if not isinstance(force, ATMMetaForce):
            raise TypeError("not an ATMMetaForce")
        return force


class NonbondedForce:
    """The parts of OpenMM's NonbondedForce that the ATM path evaluates."""

    NoCutoff, CutoffNonPeriodic, CutoffPeriodic, PME = 0, 1, 2, 4

    def __init__(self):
        h = C.c_void_p()
        call("atm_nonbonded_create", C.byref(h))
        self._h = h
        self._owned = True

    def __del__(self):
        try:
            if getattr(self, "_owned", False) and self._h:
                _lib.load().atm_nonbonded_destroy(self._h)
        except Exception:
            pass

    def addParticle(self, charge, sigma, epsilon):
        k = C.c_int()
        call("atm_nonbonded_add_particle", self._h, float(charge), float(sigma), float(epsilon), C.byref(k))
        return k.value

    def setParticleParameters(self, index, charge, sigma, epsilon):
        call("atm_nonbonded_set_particle_parameters", self._h, int(index), float(charge), float(sigma), float(epsilon))

    def getParticleParameters(self, index):
        q, s, e = C.c_double(), C.c_double(), C.c_double()
        call("atm_nonbonded_get_particle_parameters", self._h, int(index), C.byref(q), C.byref(s), C.byref(e))
        return [q.value, s.value, e.value]

    def getNumParticles(self):
        n = C.c_int()
        call("atm_nonbonded_get_num_particles", self._h, C.byref(n))
        return n.value

    def addException(self, i, j, chargeProd, sigma, epsilon):
        k = C.c_int()
        call("atm_nonbonded_add_exception", self._h, int(i), int(j), float(chargeProd), float(sigma), float(epsilon),
             C.byref(k))
        return k.value

    def getNumExceptions(self):
        n = C.c_int()
        call("atm_nonbonded_get_num_exceptions", self._h, C.byref(n))
        return n.value

    def setNonbondedMethod(self, m):
        call("atm_nonbonded_set_method", self._h, int(m))

    def setCutoffDistance(self, rc):
        call("atm_nonbonded_set_cutoff", self._h, float(rc))

    def setReactionFieldDielectric(self, e):
        call("atm_nonbonded_set_reaction_field_dielectric", self._h, float(e))

    def setEwaldErrorTolerance(self, tol):
        call("atm_nonbonded_set_ewald_error_tolerance", self._h, float(tol))

    def setPMEParameters(self, alpha, nx, ny, nz):
        call("atm_nonbonded_set_pme_parameters", self._h, float(alpha), int(nx), int(ny), int(nz))

    def setUseDispersionCorrection(self, use):
        call("atm_nonbonded_set_use_dispersion_correction", self._h, int(bool(use)))

    def setForceGroup(self, g):
        call("atm_nonbonded_set_force_group", self._h, int(g))

    def getForceGroup(self):
        g = C.c_int()
        call("atm_nonbonded_get_force_group", self._h, C.byref(g))
        return g.value


class System:
    def __init__(self):
        h = C.c_void_p()
        call("atm_system_create", C.byref(h))
        self._h = h
        self._forces = []
        self._constraints = []

    def __del__(self):
        try:
            if self._h:
                _lib.load().atm_system_destroy(self._h)
        except Exception:
            pass

    def addParticle(self, mass):
        k = C.c_int()
        call("atm_system_add_particle", self._h, float(mass), C.byref(k))
        return k.value

    def getNumParticles(self):
        n = C.c_int()
        call("atm_system_get_num_particles", self._h, C.byref(n))
        return n.value

    def setDefaultPeriodicBoxVectors(self, a, b, c):
        a, b, c = _vec3(a), _vec3(b), _vec3(c)
        call("atm_system_set_default_periodic_box_vectors", self._h, _ptr(a), _ptr(b), _ptr(c))

    def addConstraint(self, particle1, particle2, distance):
        """System::addConstraint (MD driver only; clusters of at most 4 particles)."""
        k = C.c_int()
        call("atm_system_add_constraint", self._h, int(particle1), int(particle2), float(distance), C.byref(k))
        self._constraints.append((int(particle1), int(particle2), float(distance)))
        return k.value

    def getNumConstraints(self):
        n = C.c_int()
        call("atm_system_get_num_constraints", self._h, C.byref(n))
        return n.value

    def getConstraintParameters(self, index):
        return self._constraints[index]

    def addForce(self, force):
        if isinstance(force, NonbondedForce):
            call("atm_system_add_nonbonded", self._h, force._h)
        elif isinstance(force, ATMMetaForce):
            call("atm_system_add_atm_force", self._h, force._h)
        elif hasattr(force, "_attach"):
            force._attach(self)  # bonded MD terms (atmmetaforce.md)
        else:
            raise ATMError(5, f"unsupported force type {type(force).__name__}")
        force._owned = False  # OpenMM semantics: the System owns its forces
        self._forces.append(force)
        return len(self._forces) - 1

    def getForces(self):
        return list(self._forces)


def _groups_mask(groups):
    if groups is None or (isinstance(groups, int) and groups < 0):
        return -1
    if isinstance(groups, int):
        return groups
    m = 0
    for g in groups:
        m |= 1 << int(g)
    return m


class State:
    def __init__(self, energy, forces, results):
        self._energy = energy
        self._forces = forces
        self._results = results

    def getPotentialEnergy(self):
        if self._energy is None:
            raise ATMError(3, "Invoked getPotentialEnergy() on a State which does not contain energies.")
        return self._energy

    def getForces(self, asNumpy=True):
        if self._forces is None:
            raise ATMError(3, "Invoked getForces() on a State which does not contain forces.")
        return self._forces if asNumpy else self._forces.tolist()

    def getResults(self):
        return dict(self._results)


class Context:
    """One evaluation context on one GPU.  properties: dict or 'k=v;k=v'
    (DifferencePath = 0|1)."""

    def __init__(self, system, device=0, properties=None):
        h = C.c_void_p()
        call("atm_context_create", system._h, int(device), _props(properties), C.byref(h))
        self._h = h
        self._n = system.getNumParticles()
        self._system = system

    def __del__(self):
        try:
            if self._h:
                _lib.load().atm_context_destroy(self._h)
        except Exception:
            pass

    def setPositions(self, positions):
        p = np.ascontiguousarray(np.asarray(positions, dtype=np.float64).reshape(-1, 3))
        call("atm_context_set_positions", self._h, _ptr(p), len(p))

    def setPeriodicBoxVectors(self, a, b, c):
        a, b, c = _vec3(a), _vec3(b), _vec3(c)
        call("atm_context_set_periodic_box_vectors", self._h, _ptr(a), _ptr(b), _ptr(c))

    def setParameter(self, name, value):
        call("atm_context_set_parameter", self._h, name.encode(), float(value))

    def getParameter(self, name):
        v = C.c_double()
        call("atm_context_get_parameter", self._h, name.encode(), C.byref(v))
        return v.value

    def getState(self, getEnergy=False, getForces=False, groups=-1):
        e = C.c_double()
        F = np.zeros((self._n, 3)) if getForces else None
        call("atm_context_get_state", self._h, _groups_mask(groups), C.byref(e), _ptr(F) if F is not None else None)
        r = np.zeros(NUM_RES)
        call("atm_context_get_results", self._h, _ptr(r))
        return State(e.value if getEnergy else None, F, dict(zip(RES_KEYS, r.tolist())))


def _props(p):
    if p is None:
        return None
    if isinstance(p, dict):
        p = ";".join(f"{k}={v}" for k, v in p.items())
    return p.encode()


class ReplicaBatch:
    """R replicas (any sizes) evaluated by one CUDA graph per call.
    properties as for Context; DifferencePath defaults to 1."""

    def __init__(self, systems, device=0, properties=None):
        arr = (C.c_void_p * len(systems))(*[s._h.value for s in systems])
        h = C.c_void_p()
        call("atm_batch_create", arr, len(systems), int(device), _props(properties), C.byref(h))
        self._h = h
        self._systems = list(systems)
        self.R = len(systems)
        self.n = [s.getNumParticles() for s in systems]
        self.offsets = np.concatenate([[0], np.cumsum(self.n)]).astype(int)

    def __del__(self):
        try:
            if self._h:
                _lib.load().atm_batch_destroy(self._h)
        except Exception:
            pass

    def setPositions(self, replica, positions):
        p = np.ascontiguousarray(np.asarray(positions, dtype=np.float64).reshape(-1, 3))
        if len(p) != self.n[replica]:
            raise ATMError(1, "wrong number of positions")
        call("atm_batch_set_positions", self._h, int(replica), _ptr(p))

    def setParameter(self, replica, name, value):
        call("atm_batch_set_parameter", self._h, int(replica), name.encode(), float(value))

    def setPeriodicBoxVectors(self, replica, a, b, c):
        a, b, c = _vec3(a), _vec3(b), _vec3(c)
        call("atm_batch_set_periodic_box_vectors", self._h, int(replica), _ptr(a), _ptr(b), _ptr(c))

    def evaluate(self, positions=None, forces=True, out=None, as_array=False):
        """Evaluate every replica.  positions: None (stored) or an array of
        shape (sum n, 3).  Returns (energies[R], forces[(sum n), 3] or None,
        results: list of dicts).  ``out``: a C-contiguous float64 (sum n, 3)
        array to receive the forces.  Page-locked buffers (e.g. from
        ``torch.empty(..., pin_memory=True).numpy()``) are copied to and from the
        GPU directly, without a staging copy.  ``as_array``: the results as an
        (R, NUM_RES) array (columns in ``RES_KEYS`` order) instead of dicts."""
        pos = None
        if positions is not None:
            pos = np.ascontiguousarray(np.asarray(positions, dtype=np.float64).reshape(-1, 3))
            if len(pos) != self.offsets[-1]:
                raise ATMError(1, "wrong number of positions")
        E = np.zeros(self.R)
        if out is not None:
            if out.dtype != np.float64 or not out.flags.c_contiguous or out.size != 3 * self.offsets[-1]:
                raise ATMError(1, "out must be a C-contiguous float64 array of (sum n) x 3")
            F = out
        else:
            F = np.zeros((self.offsets[-1], 3)) if forces else None
        res = np.zeros((self.R, NUM_RES))
        call("atm_batch_evaluate", self._h, _ptr(pos) if pos is not None else None, _ptr(E),
             _ptr(F) if F is not None else None, _ptr(res))
        if as_array:
            return E, F, res
        return E, F, [dict(zip(RES_KEYS, row.tolist())) for row in res]

    def results_array(self, positions=None):
        pos = None if positions is None else np.ascontiguousarray(np.asarray(positions, np.float64).reshape(-1, 3))
        res = np.zeros((self.R, NUM_RES))
        call("atm_batch_evaluate", self._h, _ptr(pos) if pos is not None else None, None, None, _ptr(res))
        return res

    def evaluateDevice(self, d_pos, d_forces, d_results, stream=0):
        """Device pointers (ints) of float64 buffers; stream a cudaStream_t (int)."""
        call("atm_batch_evaluate_device", self._h, C.c_void_p(d_pos), C.c_void_p(d_forces),
             C.c_void_p(d_results), C.c_void_p(stream))

    def setDisplacements(self, replica, displ):
        d = np.ascontiguousarray(np.asarray(displ, dtype=np.float64).reshape(-1, 3))
        if len(d) != self.n[replica]:
            raise ATMError(1, "wrong number of displacements")
        call("atm_batch_set_displacements", self._h, int(replica), _ptr(d))

    def setNonbondedParameters(self, replica, charge, sigma, epsilon):
        q, s, e = (np.ascontiguousarray(np.asarray(v, dtype=np.float64).reshape(-1)) for v in (charge, sigma, epsilon))
        if not (len(q) == len(s) == len(e) == self.n[replica]):
            raise ATMError(1, "wrong number of particle parameters")
        call("atm_batch_set_nonbonded_parameters", self._h, int(replica), _ptr(q), _ptr(s), _ptr(e))

    def backward(self, g=None):
        """Gradients of sum_r g[r] W_r (g defaults to ones) from the last
        evaluation: dict of positions, displacements (sum n, 3), charge, sigma,
        epsilon (sum n) and params (R, 5: lambda1, lambda2, alpha, u0, w0)."""
        g = np.ones(self.R) if g is None else np.ascontiguousarray(np.asarray(g, dtype=np.float64))
        N = int(self.offsets[-1])
        out = {"positions": np.zeros((N, 3)), "displacements": np.zeros((N, 3)), "charge": np.zeros(N),
               "sigma": np.zeros(N), "epsilon": np.zeros(N), "params": np.zeros((self.R, 5))}
        call("atm_batch_backward", self._h, _ptr(g), _ptr(out["positions"]), _ptr(out["displacements"]),
             _ptr(out["charge"]), _ptr(out["sigma"]), _ptr(out["epsilon"]), _ptr(out["params"]))
        return out

    def backwardDevice(self, d_g, d_dx=0, d_dd=0, d_dq=0, d_dsig=0, d_deps=0, d_dpar=0, stream=0):
        """Device-pointer variant of backward() (0 = output not wanted)."""
        call("atm_batch_backward_device", self._h, C.c_void_p(d_g), C.c_void_p(d_dx or None),
             C.c_void_p(d_dd or None), C.c_void_p(d_dq or None), C.c_void_p(d_dsig or None),
             C.c_void_p(d_deps or None), C.c_void_p(d_dpar or None), C.c_void_p(stream or None))

    def energyMatrix(self, beta=1.0):
        M = np.zeros((self.R, self.R))
        call("atm_batch_energy_matrix", self._h, float(beta), _ptr(M))
        return M

    def autotune(self, trials=5, use_cache=True):
        """Time the launch space on the stored positions and keep the fastest
        configuration; returns the report."""
        buf = C.create_string_buffer(8192)
        n = C.c_size_t()
        call("atm_batch_autotune", self._h, int(trials), int(bool(use_cache)), buf, 8192, C.byref(n))
        return buf.value.decode()

    def setProfiling(self, on):
        call("atm_batch_set_profiling", self._h, int(bool(on)))

    def kernelTimes(self):
        n = C.c_int()
        names = C.create_string_buffer(4096)
        ms = (C.c_double * 64)()
        call("atm_batch_get_kernel_times", self._h, names, 4096, ms, 64, C.byref(n))
        keys = names.value.decode().split(",") if n.value else []
        return dict(zip(keys, [ms[k] for k in range(n.value)]))

    def launchCount(self):
        n = C.c_int()
        call("atm_batch_get_launch_count", self._h, C.byref(n))
        return n.value

    def listInfo(self):
        """The pair-list skin (nm), the evaluations run and how many built the lists."""
        skin, ev, bu = C.c_double(), C.c_longlong(), C.c_longlong()
        call("atm_batch_get_list_info", self._h, C.byref(skin), C.byref(ev), C.byref(bu))
        return {"skin": skin.value, "evaluations": ev.value, "builds": bu.value}

    def stats(self):
        """Pair tiles of the last evaluation, tile rows and the largest row."""
        t, r, m = C.c_int(), C.c_int(), C.c_int()
        call("atm_batch_get_stats", self._h, C.byref(t), C.byref(r), C.byref(m))
        return {"tiles": t.value, "rows": r.value, "max_row": m.value}
