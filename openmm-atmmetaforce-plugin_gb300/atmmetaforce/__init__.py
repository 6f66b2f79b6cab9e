"""GB300-native ATMMetaForce evaluation path.

Mirrors the reference plugin's Python module ``atmmetaforce``
(python/atmmetaforceplugin.i): ``ATMMetaForce`` plus the OpenMM stand-ins the
path needs (``NonbondedForce``, ``System``, ``Context``), a ``ReplicaBatch`` for
many replicas per launch, Langevin dynamics of one or many replicas (``md``),
and (in ``autograd``) a torch.autograd.Function.
"""
import numpy as np

from ._lib import ATMError, NUM_RES, RES_KEYS
from .api import ATMMetaForce, Context, NonbondedForce, ReplicaBatch, State, System
from .md import (ATMMetaForceUtils, HarmonicAngleForce, HarmonicBondForce, LangevinIntegrator, ReplicaSimulation,
                 Simulation, md_system_from_case)

ATMMETAFORCE_VERSION = "0.3.1"


def system_from_case(case, nonbonded_group=1, atm_group=2, mass=1.0):
    """A System holding the case's NonbondedForce (in ``nonbonded_group``) and an
    ATMMetaForce over every particle (in ``atm_group``, re-evaluating
    ``nonbonded_group``), laid out as the reference's ABFE test builds it
    (python/tests/test_abfe.py:100-114).  ``mass``: one value or one per particle."""
    spec = case.spec
    sys_ = System()
    masses = [float(mass)] * case.n if np.isscalar(mass) else [float(m) for m in mass]
    for m in masses:
        sys_.addParticle(m)
    L = spec.box
    t = getattr(spec, "tilt", (0.0, 0.0, 0.0))  # reduced triclinic box vectors
    sys_.setDefaultPeriodicBoxVectors((L[0], 0, 0), (t[0], L[1], 0), (t[1], t[2], L[2]))
    nb = NonbondedForce()
    for i in range(case.n):
        nb.addParticle(spec.charge[i], spec.sigma[i], spec.epsilon[i])
    for k in range(len(spec.exc_i)):
        nb.addException(int(spec.exc_i[k]), int(spec.exc_j[k]), spec.exc_qq[k], spec.exc_sig[k], spec.exc_eps[k])
    nb.setNonbondedMethod(spec.method)
    nb.setCutoffDistance(spec.cutoff)
    nb.setReactionFieldDielectric(spec.eps_rf)
    nb.setEwaldErrorTolerance(spec.ewald_tol)
    if spec.method == NonbondedForce.PME:
        nb.setPMEParameters(spec.alpha, *spec.grid)
    nb.setUseDispersionCorrection(bool(spec.use_disp_corr))
    nb.setForceGroup(nonbonded_group)
    sys_.addForce(nb)
    p = case.params
    f = ATMMetaForce(p[0], p[1], p[2], p[3], p[4], p[5], p[6], p[7], p[8], [nonbonded_group])
    for i in range(case.n):
        d = case.displ[i]
        f.addParticle(i, d[0], d[1], d[2])
    f.setForceGroup(atm_group)
    sys_.addForce(f)
    return sys_, nb, f


__all__ = ["ATMMetaForce", "NonbondedForce", "System", "Context", "State", "ReplicaBatch", "ATMError",
           "ATMMETAFORCE_VERSION", "system_from_case", "NUM_RES", "RES_KEYS", "HarmonicBondForce",
           "HarmonicAngleForce", "ATMMetaForceUtils", "LangevinIntegrator", "ReplicaSimulation", "Simulation",
           "md_system_from_case"]
