"""The CPU oracle against golden fixtures produced by the reference's own
host-side code (tests/golden/make_golden.py): energies, forces, corrected
bond orders and the H-bond list for the fixture's positions and charges;
the charges of the reference's QEq driver; a 5-step NVE run on the
reference's QEq."""
import glob
import os

import numpy as np
import pytest

from oracle.pyoracle import Oracle

HERE = os.path.dirname(os.path.abspath(__file__))
FIXTURES = sorted(glob.glob(os.path.join(HERE, "golden", "*.npz")))
TERMS = ["e_bond", "e_ovun", "e_lp", "e_ang", "e_pen", "e_coa", "e_hb", "e_tor",
         "e_con", "e_vdW", "e_ele", "e_pol", "eng_vdwl", "eng_coul"]


def load(path):
    z = np.load(path)
    return {k: z[k] for k in z.files}


def keyset(ti, tj, im):
    return set(zip(ti.tolist(), tj.tolist(), im.tolist()))


def o_ffield(o):
    return o.ffield


@pytest.fixture(scope="module", params=FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def case(request, ffield):
    g = load(request.param)
    o = Oracle(ffield)
    o.ffield = ffield
    o.set_system(g["box"], g["x"], g["types"], g["tags"], g["q"])
    f, e = o.compute()
    return g, o, f, e


def test_fixtures_present():
    assert len(FIXTURES) >= 4


def test_energies_match_reference(case):
    g, o, f, e = case
    ref = dict(zip([str(s) for s in g["energy_names"]], g["energies"]))
    for k in TERMS:
        assert abs(e[k] - ref[k]) <= max(1e-11 * abs(ref[k]), 1e-9), (k, e[k], ref[k])


def test_forces_match_reference(case):
    g, o, f, e = case
    fr = g["forces"]
    assert np.sqrt(((f - fr) ** 2).sum() / (fr ** 2).sum()) < 1e-12


def test_bond_orders_match_reference(case):
    g, o, f, e = case
    ti, tj, im, bo = o.bond_list()
    assert keyset(ti, tj, im) == keyset(g["bond_ti"], g["bond_tj"], g["bond_img"])
    ref = {k: v for k, v in zip(zip(g["bond_ti"].tolist(), g["bond_tj"].tolist(),
                                    g["bond_img"].tolist()), g["bond_bo"])}
    for k, v in zip(zip(ti.tolist(), tj.tolist(), im.tolist()), bo):
        np.testing.assert_allclose(v, ref[k], rtol=1e-13, atol=1e-15)


def test_hbond_list_matches_reference(case):
    g, o, f, e = case
    assert keyset(*o.hbond_list()) == keyset(g["hb_ti"], g["hb_tj"], g["hb_img"])


def test_qeq_matches_reference(case):
    """Charges of the reference's own QEq driver (pre_force: init_matvec,
    CG_v2 on s and t, calculate_Q) from zero histories, and its CG
    iteration counts."""
    g, o, f, e = case
    q2 = Oracle(o_ffield(o))
    q2.set_system(g["box"], g["x"], g["types"], g["tags"], None, g["v"])
    q, its, itt = q2.qeq()
    assert (its, itt) == tuple(g["qeq_iters"])
    assert np.abs(q - g["q"]).max() <= 1e-12


def test_nve_matches_reference_qeq(case):
    """Five NVE steps whose charges came from the reference's QEq each step
    (warm s/t histories): positions, velocities, charges, forces."""
    g, o, f, e = case
    m = Oracle(o_ffield(o))
    m.set_system(g["box"], g["x"], g["types"], g["tags"], None, g["v"])
    em = m.run_nve(int(g["nve_steps"]), float(g["nve_dt"]))
    x, v, q, f5 = m.state()
    assert np.abs(x - g["nve_x"]).max() <= 1e-10
    assert np.abs(v - g["nve_v"]).max() <= 1e-10
    assert np.abs(q - g["nve_q"]).max() <= 1e-10
    fr = g["nve_f"]
    assert np.sqrt(((f5 - fr) ** 2).sum() / (fr ** 2).sum()) < 1e-9
    ref = dict(zip([str(s) for s in g["energy_names"]], g["nve_energies"]))
    for k in TERMS:
        assert abs(em[k] - ref[k]) <= max(1e-9 * abs(ref[k]), 1e-7), (k, em[k], ref[k])


def test_atom_tallies_match_reference(case):
    """Per-atom energy and virial (eflag_atom / vflag_atom) of the
    reference's ev_tally_full."""
    g, o, f, e = case
    ea, va = o.atom_tallies()
    np.testing.assert_allclose(ea, g["eatom"], rtol=1e-12, atol=1e-12)
    np.testing.assert_allclose(va, g["vatom"], rtol=1e-12, atol=1e-11)
