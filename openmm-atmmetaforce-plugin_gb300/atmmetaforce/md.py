"""Langevin dynamics of one or many ATM replicas on one GPU.

The reference drives its ATM force with OpenMM's ``LangevinIntegrator`` over
force groups {0, ATM group} (python/tests/test_abfe.py:96-103,
example/abfe/abfe.py:94-101), group 0 holding the bonded terms and the
restraints that ``ATMMetaForceUtils`` adds (python/ATMMetaForceUtils.py:79-138,
707-752).  This module mirrors those pieces over the C ABI:

  - ``HarmonicBondForce``, ``HarmonicAngleForce``: group-0 bonded terms;
  - ``ATMMetaForceUtils``: ``addVsiteRestraintForceCMCM`` and ``addPosRestraints``
    (plain floats in nm and kJ/mol instead of unit Quantities);
  - ``LangevinIntegrator(temperature, frictionCoeff, stepSize)``;
  - ``ReplicaSimulation``: R systems stepped together, one batched ATM
    evaluation per step; ``Simulation`` is the single-replica case.
"""
from __future__ import annotations

import ctypes as C

import numpy as np

from ._lib import ATMError, NUM_RES, RES_KEYS, call, load
from .api import System, _props, _ptr

KB = 0.00831446261815324  # kJ/mol/K


class HarmonicBondForce:
    """(k/2)(r - length)^2 between two particles, no periodic image."""

    def __init__(self):
        self._bonds = []
        self._system = None

    def addBond(self, particle1, particle2, length, k):
        self._bonds.append((int(particle1), int(particle2), float(length), float(k)))
        if self._system is not None:
            self._push(self._bonds[-1])
        return len(self._bonds) - 1

    def getNumBonds(self):
        return len(self._bonds)

    def getBondParameters(self, index):
        return self._bonds[index]

    def _push(self, b):
        call("atm_system_add_bond", self._system._h, b[0], b[1], b[2], b[3])

    def _attach(self, system):
        if self._system is not None:
            raise ATMError(3, "The force already belongs to a System")
        self._system = system
        for b in self._bonds:
            self._push(b)


class HarmonicAngleForce:
    """(k/2)(theta - angle)^2 at vertex particle2 (radians, kJ/mol/rad^2)."""

    def __init__(self):
        self._angles = []
        self._system = None

    def addAngle(self, particle1, particle2, particle3, angle, k):
        self._angles.append((int(particle1), int(particle2), int(particle3), float(angle), float(k)))
        if self._system is not None:
            self._push(self._angles[-1])
        return len(self._angles) - 1

    def getNumAngles(self):
        return len(self._angles)

    def getAngleParameters(self, index):
        return self._angles[index]

    def _push(self, a):
        call("atm_system_add_angle", self._system._h, a[0], a[1], a[2], a[3], a[4])

    def _attach(self, system):
        if self._system is not None:
            raise ATMError(3, "The force already belongs to a System")
        self._system = system
        for a in self._angles:
            self._push(a)


class ATMMetaForceUtils:
    """The restraint helpers of python/ATMMetaForceUtils.py on a System of this
    package.  Force constants in kJ/mol/nm^2, distances in nm."""

    def __init__(self, system):
        self.system = system

    def addVsiteRestraintForceCMCM(self, lig_cm_particles, rcpt_cm_particles, kfcm=0.0, tolcm=0.0,
                                   offset=(0.0, 0.0, 0.0)):
        """(kfcm/2) step(d - tolcm)(d - tolcm)^2, d = |c_lig - offset - c_rcpt|,
        c the mass-weighted centroids, no periodic image (ATMMetaForceUtils.py:79-138)."""
        g1 = np.ascontiguousarray(np.asarray(lig_cm_particles, dtype=np.int32))
        g2 = np.ascontiguousarray(np.asarray(rcpt_cm_particles, dtype=np.int32))
        if len(g1) == 0 or len(g2) == 0:
            raise ATMError(1, "empty centroid group")
        off = np.ascontiguousarray(np.asarray(offset, dtype=np.float64).reshape(3))
        call("atm_system_add_centroid_restraint", self.system._h, len(g1),
             g1.ctypes.data_as(C.POINTER(C.c_int)), len(g2), g2.ctypes.data_as(C.POINTER(C.c_int)),
             float(kfcm), float(tolcm), _ptr(off))

    def addPosRestraints(self, particles, refpos, fc=0.0, tol=0.0, periodic=True):
        """0.5 fc step(d - tol)(d - tol)^2 with d the (periodic) distance of each
        particle from refpos[particle] (ATMMetaForceUtils.py:707-752); refpos
        holds reference positions of every particle of the system."""
        if particles is None or len(particles) == 0:
            return
        ref = np.asarray(refpos, dtype=np.float64).reshape(-1, 3)
        call("atm_system_set_position_restraints_periodic", self.system._h, int(bool(periodic)))
        for p in particles:
            x0, y0, z0 = ref[int(p)]
            call("atm_system_add_position_restraint", self.system._h, int(p), float(x0), float(y0), float(z0),
                 float(fc), float(tol))


class LangevinIntegrator:
    """OpenMM's LangevinIntegrator (leapfrog) parameters: temperature (K),
    frictionCoeff (1/ps), stepSize (ps).  ``step(n)`` advances the simulation
    it was attached to."""

    def __init__(self, temperature, frictionCoeff, stepSize):
        self._T = float(temperature)
        self._g = float(frictionCoeff)
        self._dt = float(stepSize)
        self._seed = 0
        self._sim = None

    def getTemperature(self):
        return self._T

    def getFriction(self):
        return self._g

    def getStepSize(self):
        return self._dt

    def getRandomNumberSeed(self):
        return self._seed

    def setRandomNumberSeed(self, seed):
        if self._sim is not None:
            raise ATMError(3, "The seed is fixed once a simulation uses the integrator")
        self._seed = int(seed)

    def _update(self):
        if self._sim is not None:
            call("atm_md_set_integrator", self._sim._h, self._T, self._g, self._dt)

    def setTemperature(self, t):
        self._T = float(t)
        self._update()

    def setFriction(self, g):
        self._g = float(g)
        self._update()

    def setStepSize(self, dt):
        self._dt = float(dt)
        self._update()

    def step(self, steps):
        if self._sim is None:
            raise ATMError(3, "The integrator is not attached to a simulation")
        self._sim.step(steps)


class MDState:
    """Per replica arrays of one ``getState`` call (None where not requested)."""

    def __init__(self, positions, velocities, forces, potential, kinetic, results, offsets):
        self._x, self._v, self._f = positions, velocities, forces
        self._pe, self._ke, self._res = potential, kinetic, results
        self._off = offsets

    def _need(self, a, what):
        if a is None:
            raise ATMError(3, f"Invoked {what} on a State which does not contain it.")
        return a

    def getPositions(self, asNumpy=True):
        return self._need(self._x, "getPositions()")

    def getVelocities(self, asNumpy=True):
        return self._need(self._v, "getVelocities()")

    def getForces(self, asNumpy=True):
        return self._need(self._f, "getForces()")

    def getPotentialEnergy(self):
        return self._need(self._pe, "getPotentialEnergy()")

    def getKineticEnergy(self):
        return self._need(self._ke, "getKineticEnergy()")

    def getResults(self):
        return self._need(self._res, "getResults()")


class ReplicaSimulation:
    """R systems (each: NonbondedForce + ATMMetaForce + masses and optional
    constraints, bonded forces and restraints) stepped together on one GPU.
    properties: DifferencePath=0|1 (default 1), ReorderInterval=steps."""

    def __init__(self, systems, integrator, device=0, properties=None):
        arr = (C.c_void_p * len(systems))(*[s._h.value for s in systems])
        h = C.c_void_p()
        call("atm_md_create", arr, len(systems), int(device), _props(properties), integrator._T, integrator._g,
             integrator._dt, C.c_ulonglong(integrator._seed & ((1 << 64) - 1)), C.byref(h))
        self._h = h
        self._systems = list(systems)
        self.integrator = integrator
        integrator._sim = self
        self.R = len(systems)
        self.n = [s.getNumParticles() for s in systems]
        self.offsets = np.concatenate([[0], np.cumsum(self.n)]).astype(int)

    def __del__(self):
        try:
            if self._h:
                load().atm_md_destroy(self._h)
        except Exception:
            pass

    def _all(self, a, what):
        a = np.ascontiguousarray(np.asarray(a, dtype=np.float64).reshape(-1, 3))
        if len(a) != self.offsets[-1]:
            raise ATMError(1, f"wrong number of {what}")
        return a

    def setPositions(self, positions):
        """Positions of every replica back to back ((sum n) x 3, nm)."""
        call("atm_md_set_positions", self._h, _ptr(self._all(positions, "positions")))

    def setVelocities(self, velocities):
        call("atm_md_set_velocities", self._h, _ptr(self._all(velocities, "velocities")))

    def setVelocitiesToTemperature(self, temperature, randomSeed=0):
        call("atm_md_set_velocities_to_temperature", self._h, float(temperature),
             C.c_ulonglong(int(randomSeed) & ((1 << 64) - 1)))

    def setParameter(self, replica, name, value):
        call("atm_md_set_parameter", self._h, int(replica), name.encode(), float(value))

    def step(self, steps):
        call("atm_md_step", self._h, int(steps))

    def getState(self, getPositions=False, getVelocities=False, getForces=False, getEnergy=False):
        N = int(self.offsets[-1])
        x = np.zeros((N, 3)) if getPositions else None
        v = np.zeros((N, 3)) if getVelocities else None
        f = np.zeros((N, 3)) if getForces else None
        pe = np.zeros(self.R) if getEnergy else None
        ke = np.zeros(self.R) if getEnergy else None
        res = np.zeros((self.R, NUM_RES)) if getEnergy else None
        call("atm_md_get_state", self._h, *(_ptr(a) if a is not None else None for a in (x, v, f, pe, ke, res)))
        results = [dict(zip(RES_KEYS, r.tolist())) for r in res] if res is not None else None
        return MDState(x, v, f, pe, ke, results, self.offsets)

    def setRecording(self, interval, capacity=1024):
        """Every `interval` steps (0: off), keep on the GPU the replicas' result
        records and the R x R reduced-energy matrix at beta = 1/kT, in a ring of
        `capacity` records (no host synchronisation per step)."""
        self._rec_cap = int(capacity) if interval else 0
        call("atm_md_set_recording", self._h, int(interval), int(capacity))

    def getRecords(self):
        """The kept records, oldest first, and empties the ring: steps (n,),
        results (n, R, NUM_RES; columns in RES_KEYS order), matrices (n, R, R)."""
        cap = getattr(self, "_rec_cap", 0)
        steps = np.zeros(cap, dtype=np.int64)
        res = np.zeros((cap, self.R, NUM_RES))
        mat = np.zeros((cap, self.R, self.R))
        n = C.c_int()
        call("atm_md_get_records", self._h, steps.ctypes.data_as(C.POINTER(C.c_longlong)), _ptr(res), _ptr(mat),
             cap, C.byref(n))
        k = n.value
        return {"steps": steps[:k], "results": res[:k], "matrices": mat[:k]}

    def autotune(self, trials=20):
        """Time the evaluation's launch space and `trials` steps at each pair-list
        skin (0 to 0.2 nm), keep the fastest; returns the report.  The state is
        restored afterwards."""
        buf = C.create_string_buffer(16384)
        n = C.c_size_t()
        call("atm_md_autotune", self._h, int(trials), buf, 16384, C.byref(n))
        return buf.value.decode()

    def listInfo(self):
        """The pair-list skin (nm), the evaluations run, how many built the lists,
        and how many list checks sent the state back to their snapshot."""
        skin, ev, bu, rd = C.c_double(), C.c_longlong(), C.c_longlong(), C.c_int()
        call("atm_md_get_list_info", self._h, C.byref(skin), C.byref(ev), C.byref(bu), C.byref(rd))
        return {"skin": skin.value, "evaluations": ev.value, "builds": bu.value, "redos": rd.value}

    def info(self):
        steps, reorders = C.c_longlong(), C.c_int()
        dof = (C.c_int * self.R)()
        call("atm_md_get_info", self._h, C.byref(steps), C.byref(reorders), dof)
        return {"steps": steps.value, "reorders": reorders.value, "dof": list(dof)}

    def temperatures(self, kinetic):
        dof = np.asarray(self.info()["dof"], dtype=np.float64)
        return 2.0 * np.asarray(kinetic) / (dof * KB)


class Simulation(ReplicaSimulation):
    """One system: ``Simulation(system, integrator, device, properties)``;
    states hold that replica's arrays and scalar energies."""

    def __init__(self, system, integrator, device=0, properties=None):
        super().__init__([system], integrator, device, properties)

    def getState(self, getPositions=False, getVelocities=False, getForces=False, getEnergy=False):
        s = super().getState(getPositions, getVelocities, getForces, getEnergy)
        if getEnergy:
            s._pe, s._ke, s._res = float(s._pe[0]), float(s._ke[0]), s._res[0]
        return s


def md_system_from_case(case, terms, nonbonded_group=1, atm_group=2):
    """A System for ``ReplicaSimulation`` from a synthetic case and its MD terms
    (``synthetic.md_terms``): masses, rigid-water constraints, ligand bonds and
    angles, the receptor position restraints and the ligand-receptor centroid
    restraint, laid out as the reference's ABFE test (test_abfe.py:55-103)."""
    from . import system_from_case

    sys_, nb, f = system_from_case(case, nonbonded_group, atm_group, mass=terms.masses)
    for i, j, d in terms.constraints:
        sys_.addConstraint(int(i), int(j), float(d))
    hb = HarmonicBondForce()
    for i, j, r0, k in terms.bonds:
        hb.addBond(int(i), int(j), r0, k)
    sys_.addForce(hb)
    ha = HarmonicAngleForce()
    for i, j, l, t0, k in terms.angles:
        ha.addAngle(int(i), int(j), int(l), t0, k)
    sys_.addForce(ha)
    u = ATMMetaForceUtils(sys_)
    if len(terms.posres_particles):
        u.addPosRestraints(terms.posres_particles, terms.posres_ref, terms.posres_fc, terms.posres_tol,
                           terms.posres_periodic)
    for g1, g2, kf, tol, off in terms.centroid:
        u.addVsiteRestraintForceCMCM(g1, g2, kf, tol, off)
    return sys_, nb, f
