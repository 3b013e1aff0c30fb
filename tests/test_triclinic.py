"""Triclinic cells in the oracle (the prism box of the reference's TATB
deck, in.reaxc.lattice): zero tilts reproduce the orthogonal box exactly,
and a triclinic description of the same lattice (b' = a + b, c' = c - a + b,
i.e. tilts xy = lx, xz = -lx, yz = ly) gives the same energies, forces and
charges up to rounding, although every position is wrapped into a
different cell and every periodic image has other lattice indices."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from sw_reaxff_gb300 import systems


@pytest.fixture(scope="module")
def water():
    return systems.water_box(160, seed=5)


def solve(ffield, s, tilt):
    o = Oracle(ffield, qeq_tol=1e-12, qeq_imax=500)
    els = ["C", "H", "O", "N"]
    o.set_system(s.box, s.x, s.types(els), s.tag, None, s.v, tilt=tilt)
    q, _, _ = o.qeq()
    f, e = o.compute()
    st = o.stats()
    o.close()
    return q, f, e, st


def test_zero_tilt_is_orthogonal(ffield, water):
    a = solve(ffield, water, None)
    b = solve(ffield, water, (0.0, 0.0, 0.0))
    assert np.array_equal(a[0], b[0]) and np.array_equal(a[1], b[1])
    assert a[2] == b[2]


def test_same_lattice_triclinic_description(ffield, water):
    lx, ly, lz = water.box
    q0, f0, e0, st0 = solve(ffield, water, None)
    q1, f1, e1, st1 = solve(ffield, water, (lx, -lx, ly))
    assert st1["n_far_local"] == st0["n_far_local"]
    assert st1["n_bonds_local"] == st0["n_bonds_local"]
    assert np.abs(q1 - q0).max() < 1e-9
    assert np.sqrt(((f1 - f0) ** 2).sum() / (f0 ** 2).sum()) < 1e-9
    for k in ("e_bond", "e_ovun", "e_lp", "e_ang", "e_pen", "e_coa", "e_hb", "e_tor", "e_con",
              "e_vdW", "e_ele", "eng_vdwl", "eng_coul"):
        assert abs(e1[k] - e0[k]) <= 1e-9 * max(1.0, abs(e0[k])), k


def test_read_tatb_data():
    """The shipped TATB data file: 384 atoms (16 C6H6N6O6), box bounds and
    the "xy xz yz" tilt line (its zhi token "15.1826391451E" reads as C's
    strtod reads it)."""
    from sw_reaxff_gb300.api import DEFAULT_FFIELD
    import os
    s = systems.read_lammps_data(os.path.join(os.path.dirname(DEFAULT_FFIELD), "data.tatb"),
                                 ["C", "H", "O", "N"])
    assert s.n == 384 and s.triclinic
    assert np.allclose(s.box, [13.624, 17.1149153805, 15.1826391451])
    assert np.allclose(s.tilt, [-5.75315630927, -6.325466, 7.4257288])
    assert {e: s.elem.count(e) for e in "CHON"} == {"C": 96, "H": 96, "O": 96, "N": 96}
    r = systems.replicate(s, (2, 1, 3))
    assert r.n == 6 * 384 and np.allclose(r.tilt, [s.tilt[0], 3 * s.tilt[1], 3 * s.tilt[2]])


def test_tatb_oracle_finite(ffield):
    """The TATB crystal with the deck's control cutoffs runs through the
    oracle: finite forces that sum to zero, bonds found for every atom."""
    import os
    from sw_reaxff_gb300.api import DEFAULT_FFIELD
    s = systems.read_lammps_data(os.path.join(os.path.dirname(DEFAULT_FFIELD), "data.tatb"),
                                 ["C", "H", "O", "N"])
    o = Oracle(ffield, bond_cut=4.5, hbond_cut=6.0)
    o.set_system(s.box, s.x, s.types(["C", "H", "O", "N"]), s.tag, None, s.v, tilt=s.tilt)
    q, _, _ = o.qeq()
    f, e = o.compute()
    assert np.all(np.isfinite(f)) and abs(q.sum()) < 1e-8
    assert np.abs(f.sum(0)).max() < 1e-6 * np.abs(f).max()
    ti, _, _, _ = o.bond_list()
    assert set(ti.tolist()) == set(s.tag.tolist())
