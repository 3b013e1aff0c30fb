"""The autotuned configurations (cells of cutoff/2 or cutoff/3, 8, 16 or 32
SpMV lanes per row, the pair list built by one warp per atom or by per-cell
tiles) give the oracle's lists and forces like the default one: the pair list is equal as a set in every configuration, energies and
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


@pytest.mark.parametrize("cfg", [dict(cell_div=2, spmv_rows=8, pair_kernel=1),
                                 dict(cell_div=3, spmv_rows=16, pair_kernel=1),
                                 dict(cell_div=3, spmv_rows=32, pair_kernel=1),
                                 dict(cell_div=2, spmv_rows=16, pair_kernel=2),
                                 dict(cell_div=3, spmv_rows=8, pair_kernel=2),
                                 dict(autotune=1)])
def test_configuration_parity(ffield, ref, cfg):
    s, o, q, fo, eo = ref
    g = ReaxGPU(ffield, **cfg)
    g.set_system(s)
    qg, _, _ = g.qeq()
    st = g.stats()
    if "cell_div" in cfg:
        assert st["cell_div"] == cfg["cell_div"] and st["spmv_rows"] == cfg["spmv_rows"]
        assert st["pair_kernel"] == cfg["pair_kernel"]
    else:
        assert st["cell_div"] in (2, 3) and st["spmv_rows"] in (8, 16, 32)
        assert st["pair_kernel"] in (1, 2)
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


@pytest.mark.parametrize("seed_n", [(5, 60, 0.8), (9, 300, 0.6)], ids=["pack63", "pack305"])
def test_tiles_multi_image_boxes(ffield, seed_n):
    """Per-cell tiles on boxes below twice the cutoff (one partner at
    several images): lists bit-exact, forces at the 1e-9 bar."""
    seed, n, dens = seed_n
    s = systems.small_pack(n, dens, seed=seed)
    o = Oracle(ffield)
    o.set_system(s.box, s.x, s.types(["C", "H", "O", "N"]), s.tag, None, s.v)
    q, _, _ = o.qeq()
    fo, eo = o.compute()
    g = ReaxGPU(ffield, pair_kernel=2, autotune=0)
    g.set_box(s.box)
    g.set_atoms(s.x, s.types(g.elements), s.tag, q, s.v)
    fg, eg = g.compute()
    assert g.stats()["pair_kernel"] == 2
    assert keyset(*g.pair_list()) == keyset(*o.far_list())
    assert keyset(*g.bond_list()[:3]) == keyset(*o.bond_list()[:3])
    assert keyset(*g.hbond_list()) == keyset(*o.hbond_list())
    assert np.sqrt(((fg - fo) ** 2).sum() / (fo ** 2).sum()) < 1e-9


@pytest.mark.parametrize("precision", [0, PREC_MIXED], ids=["fp64", "mixed"])
def test_tiles_equal_warp_walk_on_a_batch(ffield, precision):
    """Many systems in one handle: the two pair-list kernels give the same
    list sizes, and charges and forces within the batch tolerance of
    test_gpu_batch.py (the row order, hence the order of the QEq sums,
    differs)."""
    S = [systems.small_pack(n, d, seed=k) for k, (n, d) in
         enumerate([(60, 0.8), (300, 0.6), (900, 0.9), (150, 0.4), (1200, 1.0)])]
    out = []
    for kern in (1, 2):
        g = ReaxGPU(ffield, precision=precision, pair_kernel=kern, autotune=0)
        g.set_systems(S)
        q, _, _ = g.qeq()
        f, _ = g.compute()
        out.append((q, f, g.stats()["n_pairs"], g.stats()["n_bonds"]))
    (q1, f1, p1, b1), (q2, f2, p2, b2) = out
    assert p1 == p2 and b1 == b2
    assert np.abs(q1 - q2).max() < 1e-5
    assert np.sqrt(((f1 - f2) ** 2).sum() / (f1 ** 2).sum()) < 1e-5
