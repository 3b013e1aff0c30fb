"""The autotuned configurations (cells of cutoff/2 or cutoff/3, 8, 16 or 32
SpMV lanes per row) give the oracle's lists and forces like the default
one: the pair list is equal as a set in every configuration, energies and
forces agree at the same charges to 1e-9, and the tuner reports what it
chose."""
import numpy as np
import pytest

from oracle.pyoracle import Oracle
from sw_reaxff_gb300 import ReaxGPU, systems
from sw_reaxff_gb300.api import PREC_MIXED

pytestmark = pytest.mark.gpu


def keyset(ti, tj, im):
    return set(zip(ti.tolist(), tj.tolist(), im.tolist()))


@pytest.fixture(scope="module")
def ref(ffield):
    s = systems.mixture(scale=0.004, seed=11)      # ~4,200 atoms, edges > 2 cutoffs
    o = Oracle(ffield)
    o.set_system(s.box, s.x, s.types(["C", "H", "O", "N"]), s.tag, None, s.v)
    q, _, _ = o.qeq()
    f, e = o.compute()
    return s, o, q, f, e


@pytest.mark.parametrize("cfg", [dict(cell_div=2, spmv_rows=8), dict(cell_div=3, spmv_rows=16),
                                 dict(cell_div=3, spmv_rows=32), dict(autotune=1)])
def test_configuration_parity(ffield, ref, cfg):
    s, o, q, fo, eo = ref
    g = ReaxGPU(ffield, **cfg)
    g.set_system(s)
    qg, _, _ = g.qeq()
    st = g.stats()
    if "cell_div" in cfg:
        assert st["cell_div"] == cfg["cell_div"] and st["spmv_rows"] == cfg["spmv_rows"]
    else:
        assert st["cell_div"] in (2, 3) and st["spmv_rows"] in (8, 16, 32)
    assert keyset(*g.pair_list()) == keyset(*o.far_list())
    assert np.abs(qg - q).max() < 1e-5
    g.set_atoms(s.x, s.types(g.elements), s.tag, q, s.v)
    fg, eg = g.compute()
    assert np.sqrt(((fg - fo) ** 2).sum() / (fo ** 2).sum()) < 1e-9
    assert abs(eg["eng_vdwl"] - eo["eng_vdwl"]) < 1e-9 * abs(eo["eng_vdwl"])


def test_mixed_cell_div3(ffield, ref):
    s, o, q, fo, _ = ref
    g = ReaxGPU(ffield, precision=PREC_MIXED, cell_div=3, spmv_rows=8)
    g.set_system(s)
    qg, _, _ = g.qeq()
    fg, _ = g.compute()
    assert keyset(*g.pair_list()) == keyset(*o.far_list())
    assert np.abs(qg - q).max() < 1e-5
    assert np.sqrt(((fg - fo) ** 2).sum() / (fo ** 2).sum()) < 1e-4
