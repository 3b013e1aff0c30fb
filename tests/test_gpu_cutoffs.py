"""FP64 form with a QEq taper radius other than the nonbonded cutoff
(qeq_swb 9 and 11 A against nonb_cut 10 A).  The pair list then reaches
max(nonb_cut, swb), H_ij is zero beyond swb and the vdW/Coulomb terms are
zero beyond nonb_cut, so the kernels take the branches a single cutoff never
reaches: H_ij by its FP64 path with the swb test (swb 9), and the
nonbonded kernel's exact cutoff test over the longer list (swb 11).
Against the oracle with the same parameters, at the parity bars: charges
within 1e-5 e; with the same charges, forces within 1e-9 relative RMS and
per-term energies within 1e-9 relative (or 1e-7 kcal/mol absolute)."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from sw_reaxff_gb300 import ReaxGPU, systems

pytestmark = pytest.mark.gpu

CASES = {
    "water600": lambda: systems.water_box(200, seed=1),
    "mixture1k": lambda: systems.mixture(scale=0.001, seed=3),
}
E_TERMS = ["e_bond", "e_hb", "e_vdW", "e_ele", "e_pol", "eng_vdwl", "eng_coul"]


@pytest.mark.parametrize("swb", [9.0, 11.0])
@pytest.mark.parametrize("case", list(CASES))
def test_qeq_cutoff_parity(ffield, case, swb):
    s = CASES[case]()
    g = ReaxGPU(ffield, qeq_swb=swb)
    g.set_system(s)
    types = s.types(g.elements)
    o = Oracle(ffield, qeq_swb=swb)
    o.set_system(s.box, s.x, types, s.tag, None, s.v)
    qo = o.qeq()[0]
    fo, eo = o.compute()
    qg = g.qeq()[0]
    assert np.abs(qg - qo).max() < 1e-5, np.abs(qg - qo).max()
    g2 = ReaxGPU(ffield, qeq_swb=swb)
    g2.set_box(s.box)
    g2.set_atoms(s.x, types, s.tag, qo, s.v)
    fg, eg = g2.compute()
    rel = np.sqrt(((fg - fo) ** 2).sum() / (fo ** 2).sum())
    assert rel < 1e-9, rel
    for t in E_TERMS:
        assert abs(eg[t] - eo[t]) <= max(1e-9 * abs(eo[t]), 1e-7), (t, eg[t], eo[t])
