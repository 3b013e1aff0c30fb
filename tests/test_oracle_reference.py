"""The oracle against the reference's own compiled host-side code, live
(only where the reference sources were available to build
oracle/_ref/libreax_ref.so; elsewhere the golden fixtures carry this
check): the force-step routines, and the QEq driver
(FixQEqReaxSunway::pre_force -> init_matvec, CG_v2 on s and t,
calculate_Q, fix_qeq_reax_sunway.cpp:539-600, 618-723, 983-1167,
1697-1755) on the same H matrix."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle, ref_available
from sw_reaxff_gb300 import systems

pytestmark = pytest.mark.skipif(not ref_available(), reason="reference build not present")

SYSTEMS = {
    "water": lambda: systems.water_box(120, seed=77),
    "mixture": lambda: systems.mixture(scale=0.0008, seed=78),
    "pack_co2": lambda: systems.small_pack(200, 0.7, seed=79),
}


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_oracle_equals_reference(name, ffield):
    s = SYSTEMS[name]()
    t = s.types(["C", "H", "O", "N"])
    o = Oracle(ffield, reference=True)
    o.set_system(s.box, s.x, t, s.tag, None, s.v)
    q, _, _ = o.qeq()
    o.set_system(s.box, s.x, t, s.tag, q, s.v)
    fo, eo = o.compute()
    _, _, _, boo = o.bond_list()
    hb_o = set(zip(*[a.tolist() for a in o.hbond_list()]))
    ea, va = o.atom_tallies()
    fr, er, bor, hb = o.ref_compute()
    ear, var = o.atom_tallies(reference=True)
    assert np.array_equal(ea, ear) and np.array_equal(va, var)
    assert np.abs(boo - bor).max() == 0.0
    assert hb_o == set(zip(*[a.tolist() for a in hb]))
    assert np.sqrt(((fo - fr) ** 2).sum() / (fr ** 2).sum()) < 1e-12
    for k in eo:
        if k == "e_pol_phys":
            continue
        assert abs(eo[k] - er[k]) <= max(1e-12 * abs(er[k]), 1e-10), (k, eo[k], er[k])


@pytest.mark.parametrize("name", list(SYSTEMS))
def test_oracle_qeq_equals_reference(name, ffield):
    """Charges, CG iteration counts and the s/t histories of the oracle's QEq
    equal the reference's own pre_force bit for bit: from zero histories,
    then along 8 NVE steps (dt 0.25 fs) whose extrapolated initial guesses
    come from the 5-deep histories."""
    s = SYSTEMS[name]()
    t = s.types(["C", "H", "O", "N"])
    a = Oracle(ffield, reference=True)
    b = Oracle(ffield, reference_qeq=True)
    for o in (a, b):
        o.set_system(s.box, s.x, t, s.tag, None, s.v)
    qa, ia, ja = a.qeq()
    qb, ib, jb = b.qeq()
    assert (ia, ja) == (ib, jb)
    assert np.array_equal(qa, qb)
    ea = a.run_nve(8, 0.25)
    eb = b.run_nve(8, 0.25)
    for x, y in zip(a.state(), b.state()):
        assert np.array_equal(x, y)
    assert ea == eb
