"""The C ABI without a GPU: symbols, host-side object model, XML and errors.

XML cases follow serialization/tests/TestSerializeATMMetaForce.cpp:12-76 of the
reference (same field values, exact equality after a round trip).
"""
import os
import re

import numpy as np
import pytest

import atmmetaforce as atm
from atmmetaforce import _lib
from atmmetaforce import synthetic as S

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADER = os.path.join(ROOT, "include", "atm_capi.h")


def declared_functions():
    txt = open(HEADER).read()
    txt = re.sub(r"/\*.*?\*/", "", txt, flags=re.S)
    return sorted(set(re.findall(r"\b(atm_[a-z0-9_]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    L = _lib.load()
    names = declared_functions()
    assert len(names) > 60
    missing = [n for n in names if not hasattr(L, n)]
    assert not missing, missing
    # and the Python binding declares a signature for each
    assert set(names) <= set(_lib.exported_names()), set(names) - set(_lib.exported_names())


def test_global_names_and_version():
    L = _lib.load()
    names = [L.atm_global_name(k).decode() for k in range(9)]
    assert names == ["ATMLambda1", "ATMLambda2", "ATMAlpha", "ATMU0", "ATMW0", "ATMUmax", "ATMUbcore", "ATMAcore",
                     "ATMDirection"]
    assert atm.ATMMetaForce.Version() == "0.3.1"
    assert atm.ATMMetaForce.Lambda1() == "ATMLambda1" and atm.ATMMetaForce.Direction() == "ATMDirection"


def test_serialization_round_trip_exact():
    f = atm.ATMMetaForce(0.0, 0.1, 0.25, 0.5, 0.6, 200.0, 100.0, 0.07, 0.0, [1])
    f.setForceGroup(30)
    f.setName("MyATMMetaForce")
    f.addParticle(0, 0.1, 0.2, 0.3)
    f.addParticle(2, 0.4, 0.5, 0.6)
    g = atm.ATMMetaForce.deserialize(f.serialize())
    assert g.getForceGroup() == 30 and g.getName() == "MyATMMetaForce"
    assert (g.getDefaultLambda1(), g.getDefaultLambda2(), g.getDefaultAlpha(), g.getDefaultU0(), g.getDefaultW0(),
            g.getDefaultUmax(), g.getDefaultUbcore(), g.getDefaultAcore(), g.getDefaultDirection()) == \
        (0.0, 0.1, 0.25, 0.5, 0.6, 200.0, 100.0, 0.07, 0.0)
    assert g.getVariableForceGroups() == [1]
    assert g.getNumParticles() == 2
    assert g.getParticleParameters(0) == [0, 0.1, 0.2, 0.3]
    assert g.getParticleParameters(1) == [2, 0.4, 0.5, 0.6]


def test_serialization_random_doubles_and_escaping():
    rng = np.random.default_rng(3)
    v = rng.normal(size=9) * 10 ** rng.uniform(-8, 8, size=9)
    f = atm.ATMMetaForce(*v, [3, 4, 7])
    f.setName('a<b & "c"')
    for k in range(50):
        f.addParticle(k, *(rng.normal(size=3) * 1e-3))
    g = atm.ATMMetaForce.deserialize(f.serialize())
    assert g.getName() == 'a<b & "c"'
    assert [g._default(k) for k in range(9)] == list(v)
    for k in range(50):
        assert g.getParticleParameters(k) == f.getParticleParameters(k)


def test_serialization_format_matches_proxy_layout():
    f = atm.ATMMetaForce(0.5, 0.5, 0.0, 0.0, 0.0, 200.0, 100.0, 0.0625, 1.0, [1])
    f.addParticle(0, 0.0, 0.0, 0.0)
    x = f.serialize()
    assert 'type="ATMMetaForce"' in x and 'version="0"' in x
    for key in ("lambda1", "lambda2", "alpha", "u0", "w0", "uMax", "ubCore", "aCore", "direction", "forceGroup",
                "name"):
        assert f' {key}="' in x
    assert "<VariableForceGroups>" in x and '<Parameter group="1"/>' in x
    assert '<Particle dx="0" dy="0" dz="0" particle="0"/>' in x


def test_deserialize_rejects_other_versions_and_bad_documents():
    f = atm.ATMMetaForce(0.5, 0.5, 0.0, 0.0, 0.0, 200.0, 100.0, 0.0625, 1.0, [1])
    x = f.serialize().replace('version="0"', 'version="1"')
    with pytest.raises(atm.ATMError) as e:
        atm.ATMMetaForce.deserialize(x)
    assert e.value.code == 7 and "Unsupported version" in str(e.value)
    with pytest.raises(atm.ATMError):
        atm.ATMMetaForce.deserialize("<Force version=\"0\" lambda1=\"0\"")
    with pytest.raises(atm.ATMError):
        atm.ATMMetaForce.deserialize(f.serialize().replace(' uMax="200"', ""))


def test_deserialize_defaults_for_optional_attributes():
    x = ('<Force version="0" lambda1="0.1" lambda2="0.2" alpha="0" u0="0" w0="0" uMax="1" ubCore="0.5" '
         'aCore="0.1" direction="1"><VariableForceGroups/><Particles/></Force>')
    g = atm.ATMMetaForce.deserialize(x)
    assert g.getForceGroup() == 0 and g.getName() == "ATMMetaForce" and g.getNumParticles() == 0


def test_particle_index_errors():
    f = atm.ATMMetaForce(0.5, 0.5, 0.0, 0.0, 0.0, 200.0, 100.0, 0.0625, 1.0, [1])
    assert f.addParticle(0) == 0
    with pytest.raises(atm.ATMError) as e:
        f.getParticleParameters(1)
    assert e.value.code == 2
    with pytest.raises(atm.ATMError):
        f.setParticleParameters(-1, 0, 0, 0, 0)
    with pytest.raises(atm.ATMError):
        f.setForceGroup(32)
    assert not f.usesPeriodicBoundaryConditions()


def test_context_rejects_atm_group_among_variable_groups():
    # ATMMetaForceImpl.cpp:75-81, checked before any device work
    c = S.water_ligand_box(300, 2.0, [4], [(1.0, 1.0, 1.0)], S.PME, 0.9, seed=1)
    sys_, nb, f = atm.system_from_case(c, nonbonded_group=1, atm_group=1)
    with pytest.raises(atm.ATMError) as e:
        atm.Context(sys_, 0)
    assert e.value.code == 8
    assert "cannot be one of the variable force groups" in str(e.value)


def test_context_requires_every_particle_in_the_force():
    c = S.water_ligand_box(300, 2.0, [4], [(1.0, 1.0, 1.0)], S.PME, 0.9, seed=1)
    sys_, nb, f = atm.system_from_case(c)
    sys_.addParticle(1.0)  # one more particle than the forces hold
    with pytest.raises(atm.ATMError) as e:
        atm.Context(sys_, 0)
    assert e.value.code in (1, 9)


def test_system_owns_added_forces():
    sys_ = atm.System()
    f = atm.ATMMetaForce(0.5, 0.5, 0.0, 0.0, 0.0, 200.0, 100.0, 0.0625, 1.0, [1])
    sys_.addForce(f)
    with pytest.raises(atm.ATMError):
        sys_.addForce(f)
    with pytest.raises(atm.ATMError):
        sys_.addForce(atm.ATMMetaForce(0.5, 0.5, 0.0, 0.0, 0.0, 200.0, 100.0, 0.0625, 1.0, [1]))
    assert _lib.load().atm_force_destroy(f._h) == 3  # owned by the System


def test_box_vectors_must_be_in_reduced_form():
    """System::setDefaultPeriodicBoxVectors accepts OpenMM's reduced triclinic
    form a = (ax,0,0), b = (bx,by,0), c = (cx,cy,cz), |bx|, |cx| <= ax/2, |cy| <= by/2."""
    s = atm.System()
    s.addParticle(1.0)
    s.setDefaultPeriodicBoxVectors((3.0, 0, 0), (1.2, 3.0, 0), (-1.4, 1.5, 3.0))  # reduced
    for a, b, c in [((3.0, 0, 0), (1.6, 3.0, 0), (0, 0, 3.0)),    # |bx| > ax/2
                    ((3.0, 0, 0), (0, 3.0, 0), (0, 1.6, 3.0)),    # |cy| > by/2
                    ((3.0, 0.1, 0), (0, 3.0, 0), (0, 0, 3.0)),    # a not along x
                    ((3.0, 0, 0), (0, 3.0, 0.2), (0, 0, 3.0))]:   # b out of the xy plane
        with pytest.raises(atm.ATMError):
            s.setDefaultPeriodicBoxVectors(a, b, c)
