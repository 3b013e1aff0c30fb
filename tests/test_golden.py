"""The CPU oracle against golden fixtures produced by the reference's own
host-side code (tests/golden/make_golden.py): energies, forces, corrected
bond orders and the H-bond list for the fixture's positions and charges."""
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


@pytest.fixture(scope="module", params=FIXTURES, ids=[os.path.basename(f)[:-4] for f in FIXTURES])
def case(request, ffield):
    g = load(request.param)
    o = Oracle(ffield)
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
