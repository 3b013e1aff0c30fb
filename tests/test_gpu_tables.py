"""FP64 form with tabulated pair functions (default) against the analytic
FP64 form: same lists, per-term energies within 1e-9 relative, forces within
1e-9 relative RMS and the same QEq charges to the CG's rounding sensitivity;
both are pinned to the oracle by the parity tests."""
import numpy as np
import pytest

from sw_reaxff_gb300 import ReaxGPU, systems

pytestmark = pytest.mark.gpu

TERMS = ["e_vdW", "e_ele", "eng_vdwl", "eng_coul", "e_bond", "e_hb", "e_pol"]


@pytest.mark.parametrize("make", [lambda: systems.water_box(200, seed=1),
                                  lambda: systems.mixture(scale=0.002, seed=4),
                                  lambda: systems.small_pack(300, 0.9, seed=7)])
def test_tabulated_equals_analytic(ffield, make):
    s = make()
    out = {}
    for tab in (0, 65536):
        g = ReaxGPU(ffield, tabulate=tab)
        assert g.table_info()[0] == tab
        g.set_system(s)
        q, _, _ = g.qeq()
        # forces at the same charges: isolate the pair-function tables from
        # the CG's sensitivity
        g2 = ReaxGPU(ffield, tabulate=tab)
        g2.set_box(s.box)
        g2.set_atoms(s.x, s.types(g.elements), s.tag, out.get("q0", q), s.v)
        f, e = g2.compute()
        out.setdefault("q0", q)
        out[tab] = (q, f, e)
    (q0, f0, e0), (q1, f1, e1) = out[0], out[65536]
    assert np.abs(q1 - q0).max() < 1e-5
    assert np.sqrt(((f1 - f0) ** 2).sum() / (f0 ** 2).sum()) < 1e-9
    for t in TERMS:
        assert abs(e1[t] - e0[t]) <= 1e-9 * max(abs(e0[t]), 1.0), t
