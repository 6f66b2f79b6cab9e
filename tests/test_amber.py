"""The prmtop reader of atmmetaforce.amber on a small hand-written topology (a
water and a four-atom chain), and, where the reference checkout is present, its
reproduction of the committed TEMOA-G1 fixture."""
import os

import numpy as np
import pytest

from atmmetaforce import amber

KCAL = 4.184


def _fmt_ints(vals, per=10, width=8):
    lines = []
    for k in range(0, len(vals), per):
        lines.append("".join(f"{v:{width}d}" for v in vals[k:k + per]))
    return lines or [""]


def _fmt_floats(vals, per=5):
    lines = []
    for k in range(0, len(vals), per):
        lines.append("".join(f"{v:16.8E}" for v in vals[k:k + per]))
    return lines or [""]


def _section(name, fmt, lines):
    return [f"%FLAG {name:<74}", f"%FORMAT({fmt})"] + lines


def _write_prmtop(path):
    sig_a, eps_kcal = 3.15, 0.636 / KCAL  # type 1: sigma 3.15 A, epsilon 0.636 kJ/mol
    A11 = 4.0 * eps_kcal * sig_a ** 12
    B11 = 4.0 * eps_kcal * sig_a ** 6
    q = [-0.834, 0.417, 0.417, 0.3, -0.2, 0.25, -0.35]
    types = [1, 2, 2, 1, 1, 1, 1]
    masses = [15.999, 1.008, 1.008, 12.011, 12.011, 12.011, 12.011]
    pointers = [7, 2] + [0] * 29
    out = ["%VERSION  VERSION_STAMP = V0001.000  DATE = 01/01/26  00:00:00"]
    out += _section("POINTERS", "10I8", _fmt_ints(pointers))
    out += _section("CHARGE", "5E16.8", _fmt_floats([x * 18.2223 for x in q]))
    out += _section("MASS", "5E16.8", _fmt_floats(masses))
    out += _section("ATOM_TYPE_INDEX", "10I8", _fmt_ints(types))
    out += _section("NONBONDED_PARM_INDEX", "10I8", _fmt_ints([1, 2, 2, 3]))
    out += _section("RESIDUE_LABEL", "20a4", ["WAT LIG "])
    out += _section("RESIDUE_POINTER", "10I8", _fmt_ints([1, 4]))
    out += _section("LENNARD_JONES_ACOEF", "5E16.8", _fmt_floats([A11, 0.0, 0.0]))
    out += _section("LENNARD_JONES_BCOEF", "5E16.8", _fmt_floats([B11, 0.0, 0.0]))
    # atom k appears as 3k in the bond/angle/dihedral lists
    out += _section("BONDS_INC_HYDROGEN", "10I8", _fmt_ints([0, 3, 1, 0, 6, 1]))
    out += _section("BONDS_WITHOUT_HYDROGEN", "10I8", _fmt_ints([9, 12, 2, 12, 15, 2, 15, 18, 2]))
    out += _section("ANGLES_INC_HYDROGEN", "10I8", _fmt_ints([3, 0, 6, 1]))
    out += _section("ANGLES_WITHOUT_HYDROGEN", "10I8", _fmt_ints([9, 12, 15, 2, 12, 15, 18, 2]))
    out += _section("DIHEDRALS_INC_HYDROGEN", "10I8", [""])
    out += _section("DIHEDRALS_WITHOUT_HYDROGEN", "10I8", _fmt_ints([9, 12, 15, 18, 1]))
    out += _section("SCEE_SCALE_FACTOR", "5E16.8", _fmt_floats([1.2]))
    out += _section("SCNB_SCALE_FACTOR", "5E16.8", _fmt_floats([2.0]))
    out += _section("BOX_DIMENSIONS", "5E16.8", _fmt_floats([90.0, 30.0, 31.0, 32.0]))
    with open(path, "w") as f:
        f.write("\n".join(out) + "\n")
    return q


def test_reader_on_a_small_topology(tmp_path):
    p = tmp_path / "mini.prmtop"
    q = _write_prmtop(p)
    prm = amber.read_prmtop(str(p))
    assert prm.natom == 7
    np.testing.assert_allclose(prm.charge, q, rtol=0, atol=1e-8)
    np.testing.assert_allclose(prm.mass, [15.999, 1.008, 1.008, 12.011, 12.011, 12.011, 12.011])
    # type 1 sigma/epsilon recovered from the A/B table; type 2 without Lennard-Jones
    np.testing.assert_allclose(prm.sigma[[0, 3, 6]], 0.315, rtol=1e-7)
    np.testing.assert_allclose(prm.epsilon[[0, 3, 6]], 0.636, rtol=1e-7)
    assert np.all(prm.epsilon[[1, 2]] == 0.0)
    assert list(prm.residue_atoms(0)) == [0, 1, 2] and list(prm.residue_atoms(1)) == [3, 4, 5, 6]
    np.testing.assert_allclose(prm.box, [3.0, 3.1, 3.2])
    pairs = {(int(i), int(j)): (qq, s, e) for i, j, qq, s, e in
             zip(prm.exc_i, prm.exc_j, prm.exc_qq, prm.exc_sig, prm.exc_eps)}
    # 1-2 and 1-3 pairs excluded outright
    for key in [(0, 1), (0, 2), (1, 2), (3, 4), (4, 5), (5, 6), (3, 5), (4, 6)]:
        assert pairs[key] == (0.0, 1.0, 0.0), key
    # the 1-4 pair scaled by SCEE 1.2 and SCNB 2.0
    qq, s, e = pairs[(3, 6)]
    assert abs(qq - q[3] * q[6] / 1.2) < 1e-9 and abs(s - 0.315) < 1e-9 and abs(e - 0.636 / 2.0) < 1e-7
    assert len(pairs) == 9


def test_system_from_prmtop_layout(tmp_path):
    p = tmp_path / "mini.prmtop"
    _write_prmtop(p)
    prm = amber.read_prmtop(str(p))
    params = [0.5, 0.5, 0.0, 0.0, 0.0, 200.0, 100.0, 0.0625, 1.0]
    sys_, nb, f = amber.system_from_prmtop(prm, prm.residue_atoms(1), (1.0, 1.0, 1.0), params)
    assert sys_.getNumParticles() == 7
    assert nb.getForceGroup() == 1 and f.getForceGroup() == 2 and f.getVariableForceGroups() == [1]
    assert list(f.getParticleParameters(4)) == [4, 1.0, 1.0, 1.0]
    assert list(f.getParticleParameters(1)) == [1, 0.0, 0.0, 0.0]


def _fixture_script():
    import importlib.util

    here = os.path.dirname(os.path.abspath(__file__))
    spec = importlib.util.spec_from_file_location("make_temoa_fixture",
                                                  os.path.join(here, "golden", "make_temoa_fixture.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_reader_reproduces_the_committed_temoa_fixture(tmp_path):
    mod = _fixture_script()
    ref = os.environ.get("ATM_REFERENCE_DIR")
    if not ref or not os.path.exists(os.path.join(ref, "python", "tests", "temoa-g1.prmtop")):
        pytest.skip("ATM_REFERENCE_DIR does not name the reference checkout the fixture was made from")
    out = tmp_path / "temoa.npz"
    mod.main(ref, str(out))
    here = os.path.dirname(os.path.abspath(__file__))
    a = np.load(os.path.join(here, "golden", "temoa_g1.npz"))
    b = np.load(out)
    assert sorted(a.files) == sorted(b.files)
    for k in a.files:
        np.testing.assert_array_equal(a[k], b[k], err_msg=k)
