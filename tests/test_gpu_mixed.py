"""Mixed-precision form (FP32 pair/bond arithmetic and FP32 QEq SpMV; FP64
positions, accumulators, CG dot products and charge sums) against the FP64
CPU oracle.  Bars from the target of the mixed form: forces within 1e-4
relative RMS, charges within 1e-5 e; per-term energies within 1e-4 relative
(or 1e-3 kcal/mol absolute); the pair, bond and H-bond lists are the FP64
lists (membership is still decided in FP64)."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from sw_reaxff_gb300 import ReaxGPU, systems
from sw_reaxff_gb300.api import PREC_MIXED

pytestmark = pytest.mark.gpu

CASES = {
    "water600": lambda: systems.water_box(200, seed=1),
    "mixture1k": lambda: systems.mixture(scale=0.001, seed=3),
    "co2pack": lambda: systems.small_pack(300, 0.6, seed=9),
}
TERMS = ["e_bond", "e_ovun", "e_lp", "e_ang", "e_pen", "e_coa", "e_hb", "e_tor",
         "e_con", "e_vdW", "e_ele", "eng_vdwl", "eng_coul"]


def keyset(ti, tj, im):
    return set(zip(ti.tolist(), tj.tolist(), im.tolist()))


@pytest.fixture(scope="module", params=list(CASES))
def run(request, ffield):
    s = CASES[request.param]()
    g = ReaxGPU(ffield, precision=PREC_MIXED)
    g.set_system(s)
    qg, its, itt = g.qeq()
    fg, eg = g.compute()
    o = Oracle(ffield)
    o.set_system(s.box, s.x, s.types(g.elements), s.tag, None, s.v)
    qo, _, _ = o.qeq()
    fo, eo = o.compute()
    # same charges on both sides for the force / energy comparison
    g2 = ReaxGPU(ffield, precision=PREC_MIXED)
    g2.set_box(s.box)
    g2.set_atoms(s.x, s.types(g.elements), s.tag, qo, s.v)
    fq, eq = g2.compute(eflag=3, vflag=4)
    return dict(s=s, g=g, g2=g2, o=o, qg=qg, qo=qo, fg=fg, eg=eg, fo=fo, eo=eo, fq=fq, eq=eq)


def test_mixed_lists_equal_fp64(run):
    assert keyset(*run["g"].pair_list()) == keyset(*run["o"].far_list())
    ti, tj, im, _ = run["g"].bond_list()
    oi, oj, om, _ = run["o"].bond_list()
    assert keyset(ti, tj, im) == keyset(oi, oj, om)
    assert keyset(*run["g"].hbond_list()) == keyset(*run["o"].hbond_list())


def test_mixed_charges(run):
    dq = np.abs(run["qg"] - run["qo"]).max()
    assert dq < 1e-5, dq
    assert abs(run["qg"].sum()) < 1e-9


def test_mixed_forces(run):
    for f in (run["fq"], run["fg"]):
        fo = run["fo"]
        rel = np.sqrt(((f - fo) ** 2).sum() / (fo ** 2).sum())
        assert rel < 1e-4, rel


def test_mixed_energies(run):
    eq, eo = run["eq"], run["eo"]
    for k in TERMS:
        assert abs(eq[k] - eo[k]) <= max(1e-4 * abs(eo[k]), 1e-3), (k, eq[k], eo[k])


def test_mixed_atom_tallies(run):
    """Per-atom energy and virial (eflag_atom / vflag_atom) of the mixed
    form against the FP64 oracle's, at the force bar."""
    ea, va = run["g2"].atom_tallies()
    eo, vo = run["o"].atom_tallies()
    assert np.sqrt(((ea - eo) ** 2).sum() / (eo ** 2).sum()) < 1e-4
    assert np.sqrt(((va - vo) ** 2).sum() / (vo ** 2).sum()) < 1e-4
